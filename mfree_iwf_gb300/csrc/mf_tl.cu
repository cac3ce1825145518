// Total-Lagrangian SPH kernels (particle_tl; rings_tl_contact rings.cpp:338-429,
// tensile_tl tensile.cpp:213-289).
//
// Set-up (once): the neighbour lists of find_neighbors (neighbor_search.h:116-147:
// every j with r^2 <= 4h^2 + eps, ascending j) are built from a cell grid whose cell
// is at least the search radius, so a 3x3 stencil is complete; each list is sorted
// ascending so the per-particle summation order is the reference's.  Then the
// Randles-Libersky correction (precomp_shape_functions.h:231-290) stores the
// corrected kernel gradient per pair.
//
// Per RK4 stage (body.h:110-123 with the action list fused):
//   k_tl_bc      Dirichlet pull on the stage state (boundary_conditions.h:36-46)
//   k_tlA        displacement gradient H (derivatives.h:101-149) and, for the rate
//                form, Fdot (derivatives.h:483-519); then per particle the velocity
//                gradient L = Fdot F^-1, continuity, EOS, Jaumann rate, Green-St
//                Venant stress and P = J F^-1 sigma (cont_mech.h, material.h)
//   k_tlB        divergence of P (derivatives.h:331-376), artificial viscosity
//                (correctors.h:83-137), momentum (cont_mech.h:70-87), advection and
//                the RK4 update (rk4.h:52-108)
#include <cub/device/device_radix_sort.cuh>

#include "mf_common.cuh"
#include "mf_kernels.h"

using namespace mfk;
using mfk_host::BodyParams;
using mfk_host::TLArgs;
using mfk_host::TLSearchArgs;
using mfk_host::TL_TILE;
using mfk_host::TL_RUN_MAX_ROWS;
using mfk_host::TL_RUN_SHIFT;

namespace MF_NS {
namespace {

enum : uint32_t {
	A_EOS = 1u << 2,
	A_ART_VISC = 1u << 6,
	A_JAUMANN = 1u << 8,
	A_CONTINUITY = 1u << 9,
	A_ADVECTION = 1u << 11,
	A_DISP = 1u << 12,
	A_GREEN = 1u << 13,
	A_C2N = 1u << 14,
	A_STRESS_TL = 1u << 15,
	A_MOMENTUM_TL = 1u << 16,
	A_VEL_TL = 1u << 17,
	A_VGRAD_TL = 1u << 18,
};

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

// ---------------------------------------------------------- neighbour search
__global__ void k_search_hash(TLSearchArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_from) return;
	const mfk_host::Geom g = a.geom[a.from_body[i]];
	uint32_t ix = (uint32_t)((a.fx[i] - g.bbmin_x) / g.dx);
	uint32_t iy = (uint32_t)((a.fy[i] - g.bbmin_y) / g.dx);
	ix = min(ix, g.nx - 1);
	iy = min(iy, g.ny - 1);
	a.keys[i] = g.cell_off + ix * g.ny + iy;
	a.vals[i] = i;
}

__global__ void k_search_cells(uint32_t n, const uint32_t* keys, uint32_t tot, uint32_t* cell_start) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k > n) return;
	if (k == n) {
		uint32_t last = (n == 0) ? 0u : keys[n - 1] + 1;
		for (uint32_t c = last; c <= tot; c++) cell_start[c] = n;
		return;
	}
	uint32_t prev = (k == 0) ? 0u : keys[k - 1] + 1;
	if (k == 0 || keys[k] != keys[k - 1])
		for (uint32_t c = prev; c <= keys[k]; c++) cell_start[c] = k;
}

// pass 0: count; pass 1: write the rows (sorted ascending) at off[i].
__global__ void k_search(TLSearchArgs a, int pass, DevStatus* st) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_to) return;
	double xi = a.tx[i], yi = a.ty[i];
	uint32_t b = a.to_body[i];
	const mfk_host::Geom g = a.geom[b];
	double h = a.h;
	double radius2 = __dmul_rn(__dmul_rn(__dmul_rn(h, h), 2.), 2.);
	double lim = __dadd_rn(radius2, a.eps);
	double box = __dadd_rn(__dmul_rn(2., h), 1e-6);  // the Manhattan predicate's half-width
	long cx = (long)floor((xi - g.bbmin_x) / g.dx), cy = (long)floor((yi - g.bbmin_y) / g.dx);
	uint32_t cnt = 0;
	uint32_t base = pass ? a.off[i] : 0u;
	for (long u = cx - 1; u <= cx + 1; u++) {
		if (u < 0 || u >= (long)g.nx) continue;
		long lo = max(cy - 1, 0l), hi = min(cy + 1, (long)g.ny - 1);
		if (lo > hi) continue;
		uint32_t c0 = g.cell_off + (uint32_t)u * g.ny + (uint32_t)lo;
		uint32_t c1 = g.cell_off + (uint32_t)u * g.ny + (uint32_t)hi + 1;
		for (uint32_t k = a.cell_start[c0]; k < a.cell_start[c1]; k++) {
			uint32_t j = a.perm[k];
			double xij = __dsub_rn(xi, a.fx[j]);
			double yij = __dsub_rn(yi, a.fy[j]);
			double r2 = __dadd_rn(__dmul_rn(xij, xij), __dmul_rn(yij, yij));
			bool in = a.manhattan ? (fabs(xij) < box && fabs(yij) < box) : (r2 <= lim);
			if (in) {
				if (pass && cnt < a.max_nbh) {
					// insertion into the ascending list
					uint32_t pos = base + cnt;
					while (pos > base && a.nbr[pos - 1] > j) {
						a.nbr[pos] = a.nbr[pos - 1];
						pos--;
					}
					a.nbr[pos] = j;
				}
				cnt++;
			}
		}
	}
	if (pass == 0) {
		a.count[i] = cnt;
		if (cnt >= a.max_nbh) raise(st, ERR_NBH_OVERFLOW, i);
		if (cnt == 0) raise(st, ERR_NO_NEIGHBOR, i);
	}
}

// ------------------------------------------------------ Randles-Libersky
// precomp_randles_libersky, precomp_shape_functions.h:231-290, FP64 always.
__global__ void k_rl(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                     const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ m,
                     const double* __restrict__ rho, const float* __restrict__ rho_f, const double* __restrict__ h,
                     double* wx, double* wy, float4* g32, DevStatus* st) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	double xi = x[i], yi = y[i], hi = h[i];
	uint32_t q0 = off[i], q1 = off[i + 1];
	double C = 0.;
	for (uint32_t q = q0; q < q1; q++) {
		uint32_t j = nbr[q];
		double rj = rho ? rho[j] : (double)rho_f[j];
		double volj = m[j] / rj;
		KR64 w = cubic_spline(xi - x[j], yi - y[j], hi);
		C += w.w * volj;
	}
	M2<double> B = M2<double>::make(0., 0., 0., 0.);
	for (uint32_t q = q0; q < q1; q++) {
		uint32_t j = nbr[q];
		double xj = x[j], yj = y[j];
		double rj = rho ? rho[j] : (double)rho_f[j];
		double volj = m[j] / rj;
		KR64 w = cubic_spline(xi - xj, yi - yj, hi);
		B.c[0][0] += (xj - xi) * w.w_x * volj * 1. / C;
		B.c[1][0] += (xj - xi) * w.w_y * volj * 1. / C;
		B.c[0][1] += (yj - yi) * w.w_x * volj * 1. / C;
		B.c[1][1] += (yj - yi) * w.w_y * volj * 1. / C;
	}
	if (!(mdet(B) != 0.) || !(C != 0.)) raise(st, ERR_SINGULAR, i);
	M2<double> invB = minverse(B);
	for (uint32_t q = q0; q < q1; q++) {
		uint32_t j = nbr[q];
		KR64 w = cubic_spline(xi - x[j], yi - y[j], hi);
		wx[q] = (w.w_x * invB.c[0][0] + w.w_y * invB.c[1][0]) * 1. / C;
		wy[q] = (w.w_x * invB.c[0][1] + w.w_y * invB.c[1][1]) * 1. / C;
	}
	// the mixed run-walk passes recompute the gradients on chip from this row's
	// correction, rounded once to FP32
	if (g32)
		g32[i] = make_float4((float)(invB.c[0][0] / C), (float)(invB.c[1][0] / C), (float)(invB.c[0][1] / C),
		                     (float)(invB.c[1][1] / C));
}

// Reference positions as float-float pairs for the run-walk passes.
__global__ void k_xf(uint32_t n, const double* __restrict__ X, const double* __restrict__ Y, float4* XF) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	FF fx = ff_split_bits(X[i]), fy = ff_split_bits(Y[i]);
	XF[i] = make_float4(fx.hi, fx.lo, fy.hi, fy.lo);
}

__global__ void k_to_float(uint64_t n, const double* a, float* b) {
	uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = (float)a[i];
}

// ------------------------------------------------------------ per stage
__global__ void k_tl_bc(TLArgs a, int on_base) {
	uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= a.n_bc) return;
	uint32_t i = a.bc_rows[r];
	double v = a.bc_v[r];
	double t = a.params[a.body_of[i]].time;
	const mfk_host::StateSoA& s = on_base ? a.base : a.st;
	s.x[i] = a.X[i] + v * t;
	s.y[i] = a.Y[i];
	s.vx[i] = v;
	s.vy[i] = 0.;
}

// The per-particle part of pass A, shared by both forms (T = double).
__device__ __forceinline__ void tl_particle(uint32_t flags, const BodyParams& pr, double Hxx, double Hxy, double Hyx,
                                            double Hyy, double Fxx, double Fxy, double Fyx, double Fyy, double rho,
                                            double Sxx, double Sxy, double Syy, double& Pxx, double& Pxy, double& Pyx,
                                            double& Pyy, double& rho_t, double& Sxx_t, double& Sxy_t, double& Syy_t) {
	double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0.;
	if (flags & A_VGRAD_TL) velocity_gradient_tl<double>(Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, vx_x, vx_y, vy_x, vy_y);
	rho_t = 0.;
	if (flags & A_CONTINUITY) rho_t = -(rho * (vx_x + vy_y));
	double p = 0.;
	if (flags & A_EOS) p = pr.c0sq * (rho - pr.rho0);
	Sxx_t = Sxy_t = Syy_t = 0.;
	if (flags & A_JAUMANN) jaumann<double>(vx_x, vx_y, vy_x, vy_y, Sxx, Sxy, Syy, pr.G, Sxx_t, Sxy_t, Syy_t);
	if (flags & A_GREEN) green_stvenant<double>(Hxx, Hxy, Hyx, Hyy, pr.D, pr.nu, Sxx, Sxy, Syy);
	Pxx = Pxy = Pyx = Pyy = 0.;
	if (flags & A_C2N) cauchy_to_nominal<double>(Hxx, Hxy, Hyx, Hyy, Sxx - p, Sxy, Syy - p, Pxx, Pxy, Pyx, Pyy);
}

// The per-row part of the mixed pass A in FP32.  GB300 issues FP64 at a small fraction
// of its FP32 rate, and in FP64 this part kept the FP64 pipe ~70 % busy, the pass's
// real bound.  FP32 suffices: F = I + H and its inverse are well conditioned, the
// density enters as rho - rho0 (the mixed state), so the EOS takes no cancellation,
// and Green-St Venant takes E from H without forming F^T F - I.
__device__ __forceinline__ void tl_particle32(uint32_t flags, const BodyParams& pr, float Hxx, float Hxy, float Hyx,
                                              float Hyy, float Fxx, float Fxy, float Fyx, float Fyy, float drho,
                                              float Sxx, float Sxy, float Syy, float& Pxx, float& Pxy, float& Pyx,
                                              float& Pyy, float& rho_t, float& Sxx_t, float& Sxy_t, float& Syy_t) {
	float vx_x = 0.f, vx_y = 0.f, vy_x = 0.f, vy_y = 0.f;
	if (flags & A_VGRAD_TL) velocity_gradient_tl<float>(Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, vx_x, vx_y, vy_x, vy_y);
	rho_t = 0.f;
	if (flags & A_CONTINUITY) rho_t = -((pr.frho0 + drho) * (vx_x + vy_y));
	float p = 0.f;
	if (flags & A_EOS) p = pr.fc0sq * drho;
	Sxx_t = Sxy_t = Syy_t = 0.f;
	if (flags & A_JAUMANN) jaumann<float>(vx_x, vx_y, vy_x, vy_y, Sxx, Sxy, Syy, pr.fG, Sxx_t, Sxy_t, Syy_t);
	if (flags & A_GREEN) green_stvenant_h<float>(Hxx, Hxy, Hyx, Hyy, pr.fD, pr.fnu, Sxx, Sxy, Syy);
	Pxx = Pxy = Pyx = Pyy = 0.f;
	if (flags & A_C2N) cauchy_to_nominal<float>(Hxx, Hxy, Hyx, Hyy, Sxx - p, Sxy, Syy - p, Pxx, Pxy, Pyx, Pyy);
}

// Sliced-ELL addressing: the 32 rows of a warp read entry k of their lists from 32
// consecutive slots, so every per-pair load of the warp is one coalesced request.
__device__ __forceinline__ uint32_t sell_base(const TLArgs& a, uint32_t i) { return a.sl_off[i >> 5] + (i & 31u); }

// ---- FP64 pass A
__global__ void __launch_bounds__(256) k_tlA64(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* sw = (const double2*)a.sw;
	uint32_t flags = a.flags;
	double uxi = s.x[i] - a.X[i], uyi = s.y[i] - a.Y[i];
	double vxi = s.vx[i], vyi = s.vy[i];
	double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
	double Fxx = 0., Fxy = 0., Fyx = 0., Fyy = 0.;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		double2 w = sw[q];
		double qwj = a.qw0[j];
		if (flags & A_DISP) {
			double uxj = s.x[j] - a.X[j], uyj = s.y[j] - a.Y[j];
			Hxx += (uxj - uxi) * w.x * qwj;
			Hxy += (uxj - uxi) * w.y * qwj;
			Hyx += (uyj - uyi) * w.x * qwj;
			Hyy += (uyj - uyi) * w.y * qwj;
		}
		if (flags & A_VEL_TL) {
			double vxj = s.vx[j], vyj = s.vy[j];
			Fxx += (vxj - vxi) * w.x * qwj;
			Fxy += (vxj - vxi) * w.y * qwj;
			Fyx += (vyj - vyi) * w.x * qwj;
			Fyy += (vyj - vyi) * w.y * qwj;
		}
	}
	const BodyParams& pr = a.params[a.body_of[i]];
	double Pxx, Pxy, Pyx, Pyy, rho_t, Sxx_t, Sxy_t, Syy_t;
	double rho = s.rho[i];
	tl_particle(flags, pr, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, rho, s.Sxx[i], s.Sxy[i], s.Syy[i], Pxx, Pxy, Pyx,
	            Pyy, rho_t, Sxx_t, Sxy_t, Syy_t);
	double* P = (double*)a.P;
	double* dA = (double*)a.dA;
	uint32_t n = a.n_total;
	P[i] = Pxx; P[n + i] = Pxy; P[2 * n + i] = Pyx; P[3 * n + i] = Pyy;
	dA[i] = rho_t; dA[n + i] = Sxx_t; dA[2 * n + i] = Sxy_t; dA[3 * n + i] = Syy_t;
	((double*)a.c)[i] = sqrt(pr.K / rho);
}

// ---- FP64 pass B + RK update
__global__ void __launch_bounds__(256) k_tlB64(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* sw = (const double2*)a.sw;
	const double* P = (const double*)a.P;
	const double* cc = (const double*)a.c;
	uint32_t n = a.n_total;
	uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[i]];
	double rho0 = pr.rho0;
	double Pxxi = P[i], Pxyi = P[n + i], Pyxi = P[2 * n + i], Pyyi = P[3 * n + i];
	double r21 = 1. / (rho0 * rho0);
	double xi = s.x[i], yi = s.y[i], vxi = s.vx[i], vyi = s.vy[i], hi = a.h[i], rhoi = s.rho[i], ci = cc[i];
	double alpha = pr.alpha, beta = pr.beta, eta = pr.eta;
	double Pxx_x = 0., Pyx_y = 0., Pxy_x = 0., Pyy_y = 0., av_x = 0., av_y = 0.;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		double2 w = sw[q];
		double mj = a.m[j];
		if (flags & A_STRESS_TL) {
			Pxx_x += mj * (Pxxi * r21 + P[j] * r21) * w.x * rho0;
			Pyx_y += mj * (Pyxi * r21 + P[2 * n + j] * r21) * w.y * rho0;
			Pxy_x += mj * (Pxyi * r21 + P[n + j] * r21) * w.x * rho0;
			Pyy_y += mj * (Pyyi * r21 + P[3 * n + j] * r21) * w.y * rho0;
		}
		if (flags & A_ART_VISC) {
			double vijx = vxi - s.vx[j], vijy = vyi - s.vy[j];
			double xij = xi - s.x[j], yij = yi - s.y[j];
			double vijposij = vijx * xij + vijy * yij;
			if (vijposij < 0.) {
				double cij = 0.5 * (ci + cc[j]);
				double hij = 0.5 * (hi + a.h[j]);
				double rhoij = 0.5 * (rhoi + s.rho[j]);
				double r2ij = xij * xij + yij * yij;
				double muij = (hij * vijposij) / (r2ij + eta * eta * hij * hij);
				double piij = (-alpha * cij * muij + beta * muij * muij) / rhoij;
				av_x += -mj * piij * w.x;
				av_y += -mj * piij * w.y;
			}
		}
	}
	const double* dA = (const double*)a.dA;
	double d[8];
	d[0] = (flags & A_ADVECTION) ? vxi : 0.;
	d[1] = (flags & A_ADVECTION) ? vyi : 0.;
	d[2] = av_x;
	d[3] = av_y;
	if (flags & A_MOMENTUM_TL) {
		d[2] += 1. / rho0 * (Pxx_x + Pyx_y) + a.fcx[i] / a.m[i];
		d[3] += 1. / rho0 * (Pxy_x + Pyy_y) + a.fcy[i] / a.m[i];
	}
	d[4] = dA[i]; d[5] = dA[n + i]; d[6] = dA[2 * n + i]; d[7] = dA[3 * n + i];
	double* bp[8] = {a.base.x, a.base.y, a.base.vx, a.base.vy, a.base.rho, a.base.Sxx, a.base.Sxy, a.base.Syy};
	double* ap[8] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy, a.acc.rho, a.acc.Sxx, a.acc.Sxy, a.acc.Syy};
	double* np[8] = {a.nxt.x, a.nxt.y, a.nxt.vx, a.nxt.vy, a.nxt.rho, a.nxt.Sxx, a.nxt.Sxy, a.nxt.Syy};
	uint32_t stg = a.stage;
	double dt = pr.dt;
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q2 = 0; q2 < 8; q2++) {
			ap[q2][i] = (stg == 0) ? d[q2] : ap[q2][i] + 2 * d[q2];
			np[q2][i] = bp[q2][i] + d[q2] * dts;  // the next stage state (ping-pong set)
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q2 = 0; q2 < 8; q2++) {
			double v = bp[q2][i] + w6 * (ap[q2][i] + d[q2]);
			bp[q2][i] = v;
			np[q2][i] = v;  // the next step's first stage starts from a copy of the particles
		}
		if (!(isfinite(bp[0][i]) && isfinite(bp[1][i]) && isfinite(bp[2][i]) && isfinite(bp[3][i])))
			raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, i);
	}
}

// ---- mixed form
// recA[i] = displacement u = x - X as float-float (16 B).
// The mixed form's per-row records for pass B (and pass A's velocities): four float4
// fields -- the nominal stress P, position and velocity as float-float pairs, and
// {h, m, rho, c} -- stored as four arrays of n_total (field f of row i at
// rec[f * n + i]).  A warp that gathers one field of 32 neighbouring rows then reads
// 512 contiguous bytes (4 cache lines) where 64-byte records would spread it over 16.
struct RecB {
	float4 P, x, v, hmrc;
};
enum { RB_P = 0, RB_X = 1, RB_V = 2, RB_H = 3 };
__device__ __forceinline__ const float4* rb_field(const void* rec, uint32_t n, int f) {
	return (const float4*)rec + (size_t)f * n;
}
__device__ __forceinline__ RecB rb_load(const void* rec, uint32_t n, uint32_t i) {
	const float4* r = (const float4*)rec;
	return RecB{r[i], r[(size_t)n + i], r[2 * (size_t)n + i], r[3 * (size_t)n + i]};
}

// End of the mixed pass A for row i: the per-row part in FP32, then the nominal stress
// into the row's record and the rate terms.
__device__ __forceinline__ void tlA_finish(const TLArgs& a, uint32_t i, float Hxx, float Hxy, float Hyx, float Hyy,
                                           float Fxx, float Fxy, float Fyx, float Fyy) {
	const mfk_host::StateSoA& s = a.st;
	const BodyParams& pr = a.params[a.body_of[i]];
	float4 P, dA;
	tl_particle32(a.flags, pr, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, s.rho_f[i], s.Sxx_f[i], s.Sxy_f[i], s.Syy_f[i],
	              P.x, P.y, P.z, P.w, dA.x, dA.y, dA.z, dA.w);
	((float4*)a.recB)[i] = P;  // field RB_P
	((float4*)a.dA32)[i] = dA;
}

// The records of row i from its state (x, y, vx, vy in FP64, rho - rho0 in FP32).
__device__ __forceinline__ void tl_pack_row(const TLArgs& a, uint32_t i, const BodyParams& pr, double x, double y,
                                            double vx, double vy, float rho_dev, void* rec) {
	FF ux = ff_split_bits(x - a.X[i]), uy = ff_split_bits(y - a.Y[i]);
	((float4*)a.recA)[i] = make_float4(ux.hi, ux.lo, uy.hi, uy.lo);
	FF fx = ff_split_bits(x), fy = ff_split_bits(y), fvx = ff_split_bits(vx), fvy = ff_split_bits(vy);
	float4* r = (float4*)rec;
	const size_t n = a.n_total;
	r[RB_X * n + i] = make_float4(fx.hi, fx.lo, fy.hi, fy.lo);
	r[RB_V * n + i] = make_float4(fvx.hi, fvx.lo, fvy.hi, fvy.lo);
	float rho = rho_dev + pr.frho0;  // the mixed state holds rho - rho0
	float K = pr.fK;
	r[RB_H * n + i] = make_float4(((const float*)a.h32)[i], ((const float*)a.m32)[i], rho, sqrtf(K / rho));
}

__global__ void k_tl_pack(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	tl_pack_row(a, i, a.params[a.body_of[i]], s.x[i], s.y[i], s.vx[i], s.vy[i], s.rho_f[i], a.recB);
}

// The same records in three parts, each as soon as its fields are in the state (a state
// arriving field by field from the host): 0 = the displacement record and the positions
// (x, y), 1 = the velocities, 2 = {h, m, rho, c} (rho).  Same values as k_tl_pack.
__global__ void k_tl_pack_part(TLArgs a, int part) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	float4* r = (float4*)a.recB;
	const size_t n = a.n_total;
	if (part == 0) {
		const double x = s.x[i], y = s.y[i];
		FF ux = ff_split_bits(x - a.X[i]), uy = ff_split_bits(y - a.Y[i]);
		((float4*)a.recA)[i] = make_float4(ux.hi, ux.lo, uy.hi, uy.lo);
		FF fx = ff_split_bits(x), fy = ff_split_bits(y);
		r[RB_X * n + i] = make_float4(fx.hi, fx.lo, fy.hi, fy.lo);
	} else if (part == 1) {
		FF fvx = ff_split_bits(s.vx[i]), fvy = ff_split_bits(s.vy[i]);
		r[RB_V * n + i] = make_float4(fvx.hi, fvx.lo, fvy.hi, fvy.lo);
	} else {
		const BodyParams& pr = a.params[a.body_of[i]];
		float rho = s.rho_f[i] + pr.frho0;
		r[RB_H * n + i] = make_float4(((const float*)a.h32)[i], ((const float*)a.m32)[i], rho, sqrtf(pr.fK / rho));
	}
}

__device__ __forceinline__ float ffd(float ahi, float alo, float bhi, float blo) { return (ahi - bhi) + (alo - blo); }

// v_ij . x_ij of a pair, FP32.  The FP32 pair passes (plain and halo tiles) share this
// and art_visc_pi with every rounding spelled out, so that neither compile can contract
// them differently: the two variants stay bit-identical.
__device__ __forceinline__ float approach(float vijx, float vijy, float xij, float yij) {
	return __fmaf_rn(vijy, yij, __fmul_rn(vijx, xij));
}

// Monaghan-Gingold viscosity Pi_ij of an approaching pair (correctors.h:83-137), FP32
// with the two divisions as reciprocal-multiply (__fdividef, 2 ulp)
__device__ __forceinline__ float art_visc_pi(float4 hmrc_i, float4 hmrc_j, float xij, float yij, float vijposij,
                                             float alpha, float beta, float eta2) {
	float cij = __fmul_rn(0.5f, __fadd_rn(hmrc_i.w, hmrc_j.w));
	float hij = __fmul_rn(0.5f, __fadd_rn(hmrc_i.x, hmrc_j.x));
	float rhoij = __fmul_rn(0.5f, __fadd_rn(hmrc_i.z, hmrc_j.z));
	float r2ij = __fmaf_rn(yij, yij, __fmul_rn(xij, xij));
	float muij = __fdividef(__fmul_rn(hij, vijposij), __fmaf_rn(__fmul_rn(eta2, hij), hij, r2ij));
	return __fdividef(__fmaf_rn(__fmul_rn(-alpha, cij), muij, __fmul_rn(__fmul_rn(beta, muij), muij)), rhoij);
}

// End of pass B for row i: momentum, advection and the RK4 update (rk4.h:52-108).
// Every load of the row is issued before the first store: the state arrays are
// distinct, but the compiler cannot know that and would otherwise wait for each load
// in turn behind the stores.  The loads stay after the pair loop (the empty asm is a
// compiler barrier): hoisted above it they would hold ~40 registers through the loop.
__device__ __forceinline__ void tlB_finish(const TLArgs& a, uint32_t i, const BodyParams& pr, float rho0, float Pxx_x,
                                           float Pyx_y, float Pxy_x, float Pyy_y, float av_x, float av_y) {
	asm volatile("" ::: "memory");
	const mfk_host::StateSoA& s = a.st;
	const uint32_t flags = a.flags, stg = a.stage;
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* np[4] = {a.nxt.x, a.nxt.y, a.nxt.vx, a.nxt.vy};
	float* bq[4] = {a.base.rho_f, a.base.Sxx_f, a.base.Sxy_f, a.base.Syy_f};
	float* aq[4] = {a.acc.rho_f, a.acc.Sxx_f, a.acc.Sxy_f, a.acc.Syy_f};
	float* nq[4] = {a.nxt.rho_f, a.nxt.Sxx_f, a.nxt.Sxy_f, a.nxt.Syy_f};
	const float4 dAi = ((const float4*)a.dA32)[i];
	const double vxs = (flags & A_ADVECTION) ? s.vx[i] : 0., vys = (flags & A_ADVECTION) ? s.vy[i] : 0.;
	// the momentum in FP32 (an FP64 division per component would keep the narrow FP64
	// pipe busy); the RK4 accumulation below stays FP64
	float fx = 0.f, fy = 0.f, inv_m = 0.f;
	if (flags & A_MOMENTUM_TL) {
		fx = (float)a.fcx[i];
		fy = (float)a.fcy[i];
		inv_m = 1.f / ((const float*)a.m32)[i];
	}
	double bv[4], av[4] = {0., 0., 0., 0.};
	float bf[4], af[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
	for (int q2 = 0; q2 < 4; q2++) {
		bv[q2] = bp[q2][i];
		bf[q2] = bq[q2][i];
		if (stg > 0) {
			av[q2] = ap[q2][i];
			af[q2] = aq[q2][i];
		}
	}
	double d[4];
	d[0] = vxs;
	d[1] = vys;
	float acc_x = av_x, acc_y = av_y;
	if (flags & A_MOMENTUM_TL) {
		acc_x += 1.f / rho0 * (Pxx_x + Pyx_y) + fx * inv_m;
		acc_y += 1.f / rho0 * (Pxy_x + Pyy_y) + fy * inv_m;
	}
	d[2] = acc_x;
	d[3] = acc_y;
	const float e[4] = {dAi.x, dAi.y, dAi.z, dAi.w};
	const double dt = pr.dt;
	double nv[4];  // the next stage's x, y, vx, vy
	float nrho;    // and its rho - rho0
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q2 = 0; q2 < 4; q2++) {
			ap[q2][i] = (stg == 0) ? d[q2] : av[q2] + 2 * d[q2];
			nv[q2] = bv[q2] + d[q2] * dts;
			np[q2][i] = nv[q2];
			aq[q2][i] = (stg == 0) ? e[q2] : af[q2] + 2.f * e[q2];
			float f = bf[q2] + e[q2] * (float)dts;
			nq[q2][i] = f;
			if (q2 == 0) nrho = f;
		}
	} else {
		double w6 = dt * 1. / 6.;
		bool ok = true;
#pragma unroll
		for (int q2 = 0; q2 < 4; q2++) {
			double v = bv[q2] + w6 * (av[q2] + d[q2]);
			bp[q2][i] = v;
			np[q2][i] = v;
			nv[q2] = v;
			ok = ok && isfinite(v);
			float f = bf[q2] + (float)w6 * (af[q2] + e[q2]);
			bq[q2][i] = f;
			nq[q2][i] = f;
			if (q2 == 0) nrho = f;
		}
		if (!ok) raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, i);
	}
	if (a.write_recs) tl_pack_row(a, i, pr, nv[0], nv[1], nv[2], nv[3], nrho, a.recB_out);
}

__global__ void __launch_bounds__(256, 8) k_tlA32(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const float2* swA = (const float2*)a.swA;
	const float4* recA = (const float4*)a.recA;
	const float4* recV = rb_field(a.recB, a.n_total, RB_V);
	uint32_t flags = a.flags;
	float4 ui = recA[i];
	float4 vi = recV[i];
	float Hxx = 0.f, Hxy = 0.f, Hyx = 0.f, Hyy = 0.f;
	float Fxx = 0.f, Fxy = 0.f, Fyx = 0.f, Fyy = 0.f;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
#pragma unroll 2
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		float2 w = swA[q];  // corrected gradient times the neighbour's quad weight
		if (flags & A_DISP) {
			float4 uj = __ldg(recA + j);
			float dux = ffd(uj.x, uj.y, ui.x, ui.y), duy = ffd(uj.z, uj.w, ui.z, ui.w);
			Hxx += dux * w.x;
			Hxy += dux * w.y;
			Hyx += duy * w.x;
			Hyy += duy * w.y;
		}
		if (flags & A_VEL_TL) {
			float4 vj = __ldg(recV + j);
			float dvx = ffd(vj.x, vj.y, vi.x, vi.y), dvy = ffd(vj.z, vj.w, vi.z, vi.w);
			Fxx += dvx * w.x;
			Fxy += dvx * w.y;
			Fyx += dvy * w.x;
			Fyy += dvy * w.y;
		}
	}
	tlA_finish(a, i, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy);
}

__global__ void __launch_bounds__(256, 5) k_tlB32(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const float2* sw = (const float2*)a.sw;
	const uint32_t n = a.n_total;
	const float4 *recP = rb_field(a.recB, n, RB_P), *recX = rb_field(a.recB, n, RB_X);
	const float4 *recV = rb_field(a.recB, n, RB_V), *recH = rb_field(a.recB, n, RB_H);
	uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[i]];
	float rho0 = pr.frho0;
	float r21 = 1.f / (rho0 * rho0);
	float sc = r21 * rho0;
	RecB ri = rb_load(a.recB, n, i);
	float alpha = pr.falpha, beta = pr.fbeta, eta2 = pr.feta2;
	float Pxx_x = 0.f, Pyx_y = 0.f, Pxy_x = 0.f, Pyy_y = 0.f, av_x = 0.f, av_y = 0.f;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
#pragma unroll 2
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		float2 w = sw[q];  // the neighbour's mass times its corrected gradient
		if (flags & A_STRESS_TL) {
			float4 Pj = __ldg(recP + j);
			float fx = sc * w.x, fy = sc * w.y;
			Pxx_x += (ri.P.x + Pj.x) * fx;
			Pyx_y += (ri.P.z + Pj.z) * fy;
			Pxy_x += (ri.P.y + Pj.y) * fx;
			Pyy_y += (ri.P.w + Pj.w) * fy;
		}
		if (flags & A_ART_VISC) {
			float4 xj = __ldg(recX + j), vj = __ldg(recV + j);
			float xij = ffd(ri.x.x, ri.x.y, xj.x, xj.y), yij = ffd(ri.x.z, ri.x.w, xj.z, xj.w);
			float vijx = ffd(ri.v.x, ri.v.y, vj.x, vj.y), vijy = ffd(ri.v.z, ri.v.w, vj.z, vj.w);
			float vijposij = approach(vijx, vijy, xij, yij);
			if (vijposij < 0.f) {
				float4 hmrc = __ldg(recH + j);
				float piij = art_visc_pi(ri.hmrc, hmrc, xij, yij, vijposij, alpha, beta, eta2);
				av_x += -piij * w.x;
				av_y += -piij * w.y;
			}
		}
	}
	tlB_finish(a, i, pr, rho0, Pxx_x, Pyx_y, Pxy_x, Pyy_y, av_x, av_y);
}

// ---- mixed form, run walk.  The same per-row arithmetic as k_tlA32 / k_tlB32 and the
// same pair order (ascending j), but with no per-pair data streamed: the neighbour
// list comes as runs of consecutive rows (one word per run, so no list entry has to
// be loaded before its neighbour's record), and each pair's corrected gradient
//     grad w_ij = invB_i grad W(X_i - X_j, h_i) / C_i      (precomp_shape_functions.h:285-287)
// is recomputed in FP32 from the float-float reference positions and the row's
// correction invB_i / C_i (rounded once from the FP64 set-up).  The weights then
// differ from the streamed FP32 ones by a few FP32 ulps.

// 10 / (7 pi) of the 2-D cubic spline (kernel.cpp:24)
constexpr float K_SPLINE_2D = 0.45472840883398667f;

// Corrected gradient of pair (i, j): the cubic spline's gradient at X_i - X_j (zero
// at r >= 2h and for r <= 1e-12, kernel.cpp:20-55) times the row's invB / C.
__device__ __forceinline__ float2 rl_grad32(float4 Xi, float4 Xj, float4 Gi, float h1, float fac) {
	float xij = ffd(Xi.x, Xi.y, Xj.x, Xj.y), yij = ffd(Xi.z, Xi.w, Xj.z, Xj.w);
	float r2 = xij * xij + yij * yij;
	float rinv = rsqrtf(fmaxf(r2, 1e-30f));
	float q = r2 * rinv * h1;
	float der = 0.f;
	if (q < 2.f && r2 > 1e-24f) {
		float t = 2.f - q;
		der = (q >= 1.f ? -0.75f * t * t : -3.0f * q * (1.f - 0.75f * q)) * h1 * rinv * fac;
	}
	float gx = xij * der, gy = yij * der;
	return make_float2(gx * Gi.x + gy * Gi.y, gx * Gi.z + gy * Gi.w);
}

// Pass A's gathers of one pair: reference position, quad weight, displacement and
// velocity records of row j.
struct PairA {
	float4 X, u, v;
	float qw;
};
__device__ __forceinline__ PairA tlA_load(const TLArgs& a, uint32_t j) {
	PairA p;
	p.X = __ldg((const float4*)a.XF + j);
	p.qw = __ldg((const float*)a.qw32 + j);
	p.u = (a.flags & A_DISP) ? __ldg((const float4*)a.recA + j) : make_float4(0.f, 0.f, 0.f, 0.f);
	p.v = (a.flags & A_VEL_TL) ? __ldg(rb_field(a.recB, a.n_total, RB_V) + j) : make_float4(0.f, 0.f, 0.f, 0.f);
	return p;
}

struct AccA {
	float Hxx = 0.f, Hxy = 0.f, Hyx = 0.f, Hyy = 0.f;
	float Fxx = 0.f, Fxy = 0.f, Fyx = 0.f, Fyy = 0.f;
};
__device__ __forceinline__ void tlA_add(uint32_t flags, const PairA& p, float4 Xi, float4 Gi, float h1, float fac,
                                        float4 ui, float4 vi, AccA& s) {
	float2 w = rl_grad32(Xi, p.X, Gi, h1, fac);
	w.x *= p.qw;  // times the neighbour's quad weight
	w.y *= p.qw;
	if (flags & A_DISP) {
		float dux = ffd(p.u.x, p.u.y, ui.x, ui.y), duy = ffd(p.u.z, p.u.w, ui.z, ui.w);
		s.Hxx += dux * w.x;
		s.Hxy += dux * w.y;
		s.Hyx += duy * w.x;
		s.Hyy += duy * w.y;
	}
	if (flags & A_VEL_TL) {
		float dvx = ffd(p.v.x, p.v.y, vi.x, vi.y), dvy = ffd(p.v.z, p.v.w, vi.z, vi.w);
		s.Fxx += dvx * w.x;
		s.Fxy += dvx * w.y;
		s.Fyx += dvy * w.x;
		s.Fyy += dvy * w.y;
	}
}

// U pairs per iteration: the gathers of both pairs are issued before either pair's
// arithmetic, and the pairs are added in list order, so U = 1 and U = 2 give the same
// bits; U = 2 keeps twice the loads in flight at the cost of registers.
// MB: blocks of 256 per SM the register budget is cut for (4: 64 registers; 5: 48,
// with spills) -- the same arithmetic, so the same results.
template <int U, int MB>
__global__ void __launch_bounds__(256, MB) k_tlA32r(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const uint32_t flags = a.flags;
	const float4 Xi = ((const float4*)a.XF)[i], Gi = ((const float4*)a.G)[i];
	const float h1 = 1.f / ((const float*)a.h32)[i], fac = K_SPLINE_2D * h1 * h1;
	const float4 ui = ((const float4*)a.recA)[i];
	const float4 vi = rb_field(a.recB, a.n_total, RB_V)[i];
	AccA s;
	uint32_t q = a.r_sl[i >> 5] + (i & 31u), nr = a.r_cnt[i];
	for (uint32_t r = 0; r < nr; r++, q += 32) {
		const uint32_t run = a.runs[q];
		const uint32_t j0 = run & (TL_RUN_MAX_ROWS - 1u), j1 = j0 + (run >> TL_RUN_SHIFT) + 1u;
		if (U == 1) {
			for (uint32_t j = j0; j < j1; j++) tlA_add(flags, tlA_load(a, j), Xi, Gi, h1, fac, ui, vi, s);
		} else {
			for (uint32_t j = j0; j < j1; j += 2) {
				const bool two = j + 1 < j1;
				const PairA p0 = tlA_load(a, j), p1 = tlA_load(a, two ? j + 1 : j);
				tlA_add(flags, p0, Xi, Gi, h1, fac, ui, vi, s);
				if (two) tlA_add(flags, p1, Xi, Gi, h1, fac, ui, vi, s);
			}
		}
	}
	tlA_finish(a, i, s.Hxx, s.Hxy, s.Hyx, s.Hyy, s.Fxx, s.Fxy, s.Fyx, s.Fyy);
}

// Pass B's gathers of one pair: row j's record and reference position.
struct PairB {
	float4 P, x, v, hmrc, X;
};
__device__ __forceinline__ PairB tlB_load(const TLArgs& a, uint32_t j) {
	const uint32_t n = a.n_total;
	PairB p;
	p.hmrc = __ldg(rb_field(a.recB, n, RB_H) + j);
	p.X = __ldg((const float4*)a.XF + j);
	p.P = (a.flags & A_STRESS_TL) ? __ldg(rb_field(a.recB, n, RB_P) + j) : make_float4(0.f, 0.f, 0.f, 0.f);
	if (a.flags & A_ART_VISC) {
		p.x = __ldg(rb_field(a.recB, n, RB_X) + j);
		p.v = __ldg(rb_field(a.recB, n, RB_V) + j);
	} else {
		p.x = p.v = make_float4(0.f, 0.f, 0.f, 0.f);
	}
	return p;
}

struct AccB {
	float Pxx_x = 0.f, Pyx_y = 0.f, Pxy_x = 0.f, Pyy_y = 0.f, av_x = 0.f, av_y = 0.f;
};
__device__ __forceinline__ void tlB_add(uint32_t flags, const PairB& p, const RecB& ri, float4 Xi, float4 Gi, float h1,
                                        float fac, float sc, float alpha, float beta, float eta2, AccB& s) {
	float2 w = rl_grad32(Xi, p.X, Gi, h1, fac);
	w.x *= p.hmrc.y;  // times the neighbour's mass
	w.y *= p.hmrc.y;
	if (flags & A_STRESS_TL) {
		float fx = sc * w.x, fy = sc * w.y;
		s.Pxx_x += (ri.P.x + p.P.x) * fx;
		s.Pyx_y += (ri.P.z + p.P.z) * fy;
		s.Pxy_x += (ri.P.y + p.P.y) * fx;
		s.Pyy_y += (ri.P.w + p.P.w) * fy;
	}
	if (flags & A_ART_VISC) {
		float xij = ffd(ri.x.x, ri.x.y, p.x.x, p.x.y), yij = ffd(ri.x.z, ri.x.w, p.x.z, p.x.w);
		float vijx = ffd(ri.v.x, ri.v.y, p.v.x, p.v.y), vijy = ffd(ri.v.z, ri.v.w, p.v.z, p.v.w);
		float vijposij = approach(vijx, vijy, xij, yij);
		if (vijposij < 0.f) {
			float piij = art_visc_pi(ri.hmrc, p.hmrc, xij, yij, vijposij, alpha, beta, eta2);
			s.av_x += -piij * w.x;
			s.av_y += -piij * w.y;
		}
	}
}

// MB: blocks of 256 per SM the register budget is cut for (3: 72 registers; 4: 64,
// with a few bytes of spills) -- the same arithmetic, so the same results.
template <int U, int MB>
__global__ void __launch_bounds__(256, MB) k_tlB32r(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[i]];
	const float rho0 = pr.frho0;
	const float r21 = 1.f / (rho0 * rho0);
	const float sc = r21 * rho0;
	const RecB ri = rb_load(a.recB, a.n_total, i);
	const float4 Xi = ((const float4*)a.XF)[i], Gi = ((const float4*)a.G)[i];
	const float h1 = 1.f / ri.hmrc.x, fac = K_SPLINE_2D * h1 * h1;
	const float alpha = pr.falpha, beta = pr.fbeta, eta2 = pr.feta2;
	AccB s;
	uint32_t q = a.r_sl[i >> 5] + (i & 31u), nr = a.r_cnt[i];
	for (uint32_t r = 0; r < nr; r++, q += 32) {
		const uint32_t run = a.runs[q];
		const uint32_t j0 = run & (TL_RUN_MAX_ROWS - 1u), j1 = j0 + (run >> TL_RUN_SHIFT) + 1u;
		if (U == 1) {
			for (uint32_t j = j0; j < j1; j++)
				tlB_add(flags, tlB_load(a, j), ri, Xi, Gi, h1, fac, sc, alpha, beta, eta2, s);
		} else {
			for (uint32_t j = j0; j < j1; j += 2) {
				const bool two = j + 1 < j1;
				const PairB p0 = tlB_load(a, j), p1 = tlB_load(a, two ? j + 1 : j);
				tlB_add(flags, p0, ri, Xi, Gi, h1, fac, sc, alpha, beta, eta2, s);
				if (two) tlB_add(flags, p1, ri, Xi, Gi, h1, fac, sc, alpha, beta, eta2, s);
			}
		}
	}
	tlB_finish(a, i, pr, rho0, s.Pxx_x, s.Pyx_y, s.Pxy_x, s.Pyy_y, s.av_x, s.av_y);
}

// ---- mixed form over halo tiles.  The same per-row arithmetic, in the same order, as
// k_tlA32 / k_tlB32 (so the results are bit-identical); the neighbours' records come
// from shared memory, where the block first copies its tile's halo (a compact 2-D
// patch of 128 rows names ~250 distinct rows, against ~2,700 list entries) with
// 16-byte cp.async copies, all in flight at once, instead of one scattered global
// load per list entry.  The lists (halo slot + weights) stream from global memory.
__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
	uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_wait_all() {
	asm volatile("cp.async.commit_group;\n" ::: "memory");
	asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(TL_TILE) k_tlA32t(TLArgs a) {
	extern __shared__ float4 smA[];  // [halo_max] u, then [halo_max] v
	const uint32_t t = blockIdx.x, HM = a.halo_max;
	const uint32_t h0 = a.t_halo_off[t], hn = a.t_halo_off[t + 1] - h0;
	const float4* recA = (const float4*)a.recA;
	const float4* rec4 = (const float4*)a.recB;
	for (uint32_t e = threadIdx.x; e < 2 * hn; e += TL_TILE) {
		uint32_t s_ = e >> 1, j = a.t_halo[h0 + s_];
		cp16(smA + (e & 1u) * HM + s_, (e & 1u) ? rec4 + (size_t)RB_V * a.n_total + j : recA + j);  // u, or v
	}
	const uint32_t p = t * TL_TILE + threadIdx.x;
	const bool live = p < a.n_total;
	const uint32_t i = live ? a.t_rows[p] : 0u;
	const float4 ui = recA[i];
	const float4 vi = rec4[(size_t)RB_V * a.n_total + i];
	const uint32_t c = live ? a.t_cnt[p] : 0u;
	cp_wait_all();
	__syncthreads();
	if (!live) return;
	const mfk_host::StateSoA& s = a.st;
	const float2* swA = (const float2*)a.t_swA;
	const uint32_t flags = a.flags;
	float Hxx = 0.f, Hxy = 0.f, Hyx = 0.f, Hyy = 0.f;
	float Fxx = 0.f, Fxy = 0.f, Fyx = 0.f, Fyy = 0.f;
	uint32_t q = a.t_sl[p >> 5] + (p & 31u);
#pragma unroll 4
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t l = __ldg(a.t_loc + q);
		float2 w = __ldg(swA + q);
		if (flags & A_DISP) {
			float4 uj = smA[l];
			float dux = ffd(uj.x, uj.y, ui.x, ui.y), duy = ffd(uj.z, uj.w, ui.z, ui.w);
			Hxx += dux * w.x;
			Hxy += dux * w.y;
			Hyx += duy * w.x;
			Hyy += duy * w.y;
		}
		if (flags & A_VEL_TL) {
			float4 vj = smA[HM + l];
			float dvx = ffd(vj.x, vj.y, vi.x, vi.y), dvy = ffd(vj.z, vj.w, vi.z, vi.w);
			Fxx += dvx * w.x;
			Fxy += dvx * w.y;
			Fyx += dvy * w.x;
			Fyy += dvy * w.y;
		}
	}
	tlA_finish(a, i, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy);
}

__global__ void __launch_bounds__(TL_TILE, 8) k_tlB32t(TLArgs a) {
	extern __shared__ float4 smB[];  // RecB fields as four arrays of halo_max: P, x, v, hmrc
	const uint32_t t = blockIdx.x, HM = a.halo_max;
	const uint32_t h0 = a.t_halo_off[t], hn = a.t_halo_off[t + 1] - h0;
	const float4* rec4 = (const float4*)a.recB;
	for (uint32_t e = threadIdx.x; e < 4 * hn; e += TL_TILE) {
		uint32_t s_ = e >> 2, f = e & 3u;  // four threads copy one row's four fields
		cp16(smB + f * HM + s_, rec4 + (size_t)f * a.n_total + a.t_halo[h0 + s_]);
	}
	// this row's own data, requested while the copies are in flight
	const uint32_t p = t * TL_TILE + threadIdx.x;
	const bool live = p < a.n_total;
	const uint32_t i = live ? a.t_rows[p] : 0u;
	const RecB ri = rb_load(a.recB, a.n_total, i);
	const uint32_t c = live ? a.t_cnt[p] : 0u;
	const uint32_t bi = a.body_of[i];
	cp_wait_all();
	__syncthreads();
	if (!live) return;
	const mfk_host::StateSoA& s = a.st;
	const float2* sw = (const float2*)a.t_sw;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[bi];
	float rho0 = pr.frho0;
	float r21 = 1.f / (rho0 * rho0);
	float sc = r21 * rho0;
	float alpha = pr.falpha, beta = pr.fbeta, eta2 = pr.feta2;
	float Pxx_x = 0.f, Pyx_y = 0.f, Pxy_x = 0.f, Pyy_y = 0.f, av_x = 0.f, av_y = 0.f;
	uint32_t q = a.t_sl[p >> 5] + (p & 31u);
#pragma unroll 4
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t l = __ldg(a.t_loc + q);
		float2 w = __ldg(sw + q);  // the neighbour's mass times its corrected gradient
		if (flags & A_STRESS_TL) {
			float4 Pj = smB[l];
			float fx = sc * w.x, fy = sc * w.y;
			Pxx_x += (ri.P.x + Pj.x) * fx;
			Pyx_y += (ri.P.z + Pj.z) * fy;
			Pxy_x += (ri.P.y + Pj.y) * fx;
			Pyy_y += (ri.P.w + Pj.w) * fy;
		}
		if (flags & A_ART_VISC) {
			float4 xj = smB[HM + l], vj = smB[2 * HM + l];
			float xij = ffd(ri.x.x, ri.x.y, xj.x, xj.y), yij = ffd(ri.x.z, ri.x.w, xj.z, xj.w);
			float vijx = ffd(ri.v.x, ri.v.y, vj.x, vj.y), vijy = ffd(ri.v.z, ri.v.w, vj.z, vj.w);
			float vijposij = approach(vijx, vijy, xij, yij);
			if (vijposij < 0.f) {
				float4 hmrc = smB[3 * HM + l];
				float piij = art_visc_pi(ri.hmrc, hmrc, xij, yij, vijposij, alpha, beta, eta2);
				av_x += -piij * w.x;
				av_y += -piij * w.y;
			}
		}
	}
	tlB_finish(a, i, pr, rho0, Pxx_x, Pyx_y, Pxy_x, Pyy_y, av_x, av_y);
}

// Sliced ELL over tile positions: the weights of row t_rows[p] copied from the row-order
// sliced ELL (the halo slots, t_loc, come from the host).
__global__ void k_tile_sell(uint32_t n, const uint32_t* __restrict__ t_rows, const uint32_t* __restrict__ sl_off,
                            const uint16_t* __restrict__ cnt, const float2* __restrict__ sw, const float2* __restrict__ swA,
                            const uint32_t* __restrict__ t_sl, uint16_t* t_cnt, float2* t_sw, float2* t_swA) {
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= n) return;
	uint32_t i = t_rows[p];
	uint32_t c = cnt[i];
	t_cnt[p] = (uint16_t)c;
	uint32_t qo = sl_off[i >> 5] + (i & 31u), qn = t_sl[p >> 5] + (p & 31u);
	for (uint32_t k = 0; k < c; k++, qo += 32, qn += 32) {
		t_sw[qn] = sw[qo];
		t_swA[qn] = swA[qo];
	}
}

// CSR (set-up order) -> sliced ELL; the mixed form gets FP32 gradients pre-multiplied
// by the neighbour's mass (pass B) and by its quad weight (pass A), in FP64 then rounded.
__global__ void k_to_sell(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                          const double* __restrict__ wx, const double* __restrict__ wy, const uint32_t* __restrict__ sl_off,
                          uint16_t* cnt, uint32_t* snbr, double2* sw64, float2* sw32, float2* swA32,
                          const double* __restrict__ qw, const double* __restrict__ mass) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t base = sl_off[i >> 5] + (i & 31u);
	uint32_t q0 = off[i], c = off[i + 1] - q0;
	cnt[i] = (uint16_t)c;
	for (uint32_t k = 0; k < c; k++) {
		uint32_t q = base + 32 * k;
		uint32_t j = nbr[q0 + k];
		snbr[q] = j;
		double gx = wx[q0 + k], gy = wy[q0 + k];
		if (sw64) sw64[q] = make_double2(gx, gy);
		if (sw32) sw32[q] = make_float2((float)(gx * mass[j]), (float)(gy * mass[j]));
		if (swA32) swA32[q] = make_float2((float)(gx * qw[j]), (float)(gy * qw[j]));
	}
}

__global__ void k_advance_time(uint32_t nb, BodyParams* P) {
	uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b < nb) P[b].time += P[b].dt;
}

}  // namespace

cudaError_t tl_search(const TLSearchArgs& a, int pass, cudaStream_t s) {
	DevStatus* st = reinterpret_cast<DevStatus*>(a.status);
	if (pass == 0) {
		k_search_hash<<<grid1(a.n_from, 256), 256, 0, s>>>(a);
		size_t tmp = a.sort_tmp_bytes;
		cudaError_t e = cub::DeviceRadixSort::SortPairs(a.sort_tmp, tmp, a.keys, a.keys_sorted, a.vals, a.perm,
		                                                (int)a.n_from, 0, a.sort_bits, s);
		if (e != cudaSuccess) return e;
		k_search_cells<<<grid1(a.n_from + 1, 256), 256, 0, s>>>(a.n_from, a.keys_sorted, a.total_cells, a.cell_start);
	}
	k_search<<<grid1(a.n_to, 128), 128, 0, s>>>(a, pass, st);
	return cudaGetLastError();
}

size_t tl_sort_tmp_bytes(uint32_t n, int bits) {
	size_t bytes = 0;
	cub::DeviceRadixSort::SortPairs(nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
	                                (uint32_t*)nullptr, (int)n, 0, bits);
	return bytes;
}

cudaError_t tl_rl(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* x, const double* y,
                  const double* m, const double* rho, const float* rho_f, const double* h, double* wx, double* wy,
                  void* g32, void* status, cudaStream_t s) {
	k_rl<<<grid1(n, 128), 128, 0, s>>>(n, off, nbr, x, y, m, rho, rho_f, h, wx, wy, (float4*)g32,
	                                   reinterpret_cast<DevStatus*>(status));
	return cudaGetLastError();
}

cudaError_t tl_ref_positions(uint32_t n, const double* X, const double* Y, void* XF, cudaStream_t s) {
	if (n) k_xf<<<grid1(n, 256), 256, 0, s>>>(n, X, Y, (float4*)XF);
	return cudaGetLastError();
}

cudaError_t to_float(uint64_t n, const double* a, float* b, cudaStream_t s) {
	k_to_float<<<grid1(n, 256), 256, 0, s>>>(n, a, b);
	return cudaGetLastError();
}

cudaError_t tl_to_sell(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* wx, const double* wy,
                       const uint32_t* sl_off, uint16_t* cnt, uint32_t* snbr, void* sw64, void* sw32, void* swA32,
                       const double* qw, const double* mass, cudaStream_t s) {
	k_to_sell<<<grid1(n, 128), 128, 0, s>>>(n, off, nbr, wx, wy, sl_off, cnt, snbr, (double2*)sw64, (float2*)sw32,
	                                        (float2*)swA32, qw, mass);
	return cudaGetLastError();
}

cudaError_t tl_tile_sell(uint32_t n, const uint32_t* t_rows, const uint32_t* sl_off, const uint16_t* cnt, const void* sw,
                         const void* swA, const uint32_t* t_sl, uint16_t* t_cnt, void* t_sw, void* t_swA, cudaStream_t s) {
	k_tile_sell<<<grid1(n, 256), 256, 0, s>>>(n, t_rows, sl_off, cnt, (const float2*)sw, (const float2*)swA, t_sl, t_cnt,
	                                          (float2*)t_sw, (float2*)t_swA);
	return cudaGetLastError();
}

// dynamic shared memory of the tiled passes: the halo records, 32 B (pass A) / 64 B
// (pass B) per halo row
size_t tl_tile_smem(int pass, uint32_t halo_max, uint32_t /*ent_max*/) {
	return (pass == 0 ? 2 : 4) * (size_t)halo_max * sizeof(float4);
}

cudaError_t tl_tile_attrs(uint32_t halo_max, uint32_t ent_max) {
	cudaError_t e = cudaFuncSetAttribute(k_tlA32t, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     (int)tl_tile_smem(0, halo_max, ent_max));
	if (e != cudaSuccess) return e;
	return cudaFuncSetAttribute(k_tlB32t, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                            (int)tl_tile_smem(1, halo_max, ent_max));
}

cudaError_t tl_stage(const TLArgs& a, bool mixed, int part, cudaStream_t s) {
	// part 0: BCs on the stage state, 1: pack (mixed), 2: pass A, 3: pass B,
	// 4: BCs on the particles after the combine, 5: advance the body clocks,
	// 6-8: pack one part of the records (mixed)
	switch (part) {
	case 0:
		if (a.n_bc) k_tl_bc<<<grid1(a.n_bc, 128), 128, 0, s>>>(a, 0);
		break;
	case 1:
		if (mixed) k_tl_pack<<<grid1(a.n_total, 256), 256, 0, s>>>(a);
		break;
	case 2: {
		unsigned bs = a.block ? a.block : 128;
		if (mixed && a.t_rows) k_tlA32t<<<a.n_tiles, TL_TILE, tl_tile_smem(0, a.halo_max, a.t_ent_max), s>>>(a);
		else if (mixed && a.runs && a.unroll == 2) k_tlA32r<2, 3><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed && a.runs && a.unroll == 4) k_tlA32r<1, 5><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed && a.runs) k_tlA32r<1, 4><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed) k_tlA32<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else k_tlA64<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		break;
	}
	case 3: {
		unsigned bs = a.block ? a.block : 128;
		if (mixed && a.t_rows) k_tlB32t<<<a.n_tiles, TL_TILE, tl_tile_smem(1, a.halo_max, a.t_ent_max), s>>>(a);
		else if (mixed && a.runs && a.unroll == 2) k_tlB32r<2, 2><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed && a.runs && (a.unroll == 3 || a.unroll == 4)) k_tlB32r<1, 4><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed && a.runs) k_tlB32r<1, 3><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else if (mixed) k_tlB32<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else k_tlB64<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		break;
	}
	case 4:
		if (a.n_bc) k_tl_bc<<<grid1(a.n_bc, 128), 128, 0, s>>>(a, 1);
		break;
	case 5:
		k_advance_time<<<grid1(a.n_bodies, 128), 128, 0, s>>>(a.n_bodies, const_cast<BodyParams*>(a.params));
		break;
	case 6:
	case 7:
	case 8:  // the records' positions, velocities, {h, m, rho, c} (mixed)
		if (mixed) k_tl_pack_part<<<grid1(a.n_total, 256), 256, 0, s>>>(a, part - 6);
		break;
	}
	return cudaGetLastError();
}

}  // namespace MF_NS
