// Corotational SPH (particle_corotational; rings_corot_contact rings.cpp:245-336,
// tensile_corot tensile.cpp:137-211): total-Lagrangian neighbour lists with plain SPH
// weights, and a per-particle rotation that takes the neighbourhood's rigid rotation
// out of the displacement gradient.
//
// Set-up (once): find_neighbors (shared with the TL path), then precomp_sph
// (precomp_shape_functions.h:210-229): W and grad W of every listed pair from the
// set-up positions, stored per pair in the sliced-ELL layout.
//
// Per RK4 stage (body.h:110-123, the action list fused):
//   k_crR   corotational_anisotropy_tensor (corotational.h:32-84): the rotation R_i
//           from the angle of sum_j (x_j - x_i)(X_j - X_i)^T m_j W_ij
//   k_crA   derive_displacement_corotational (derivatives.h:202-258), then per particle
//           material_compute_stress_cauchy_green (material.h:102-130) and
//           contmech_cauchy_to_nominal (cont_mech.h:154-169)
//   k_crB   derive_stress_corotational (derivatives.h:521-588) with the contact force,
//           correctors_mghn_artificial_viscosity (correctors.h:83-137) added pair by
//           pair onto that velocity rate as the reference does, contmech_advection,
//           and the RK4 update (rk4.h:52-108)
//
// Elastic-potential SPH (particle_potential; rings_potential_contact rings.cpp:431-520,
// tensile_potential tensile.cpp:291-361, rotation_potential rotation.cpp:212-272) runs
// on the same lists with the symmetric Randles-Libersky weights
// (precomp_shape_functions.h:292-315: per pair also the gradient that j's list holds
// for i, found once at set-up by k_sell_wji):
//   k_ptA   derive_displacement (derivatives.h:101-149), Green-St Venant stress
//           (material.h:132-161) and per particle F_e = -2 V F S (potential.h:43-48)
//   k_crB   (potential form) f_ij = F_e,i grad W_ij, f_ji = F_e,j grad W_ji summed as
//           0.5 (f_ji - f_ij) / m_i (potential.h:50-76), the contact force, then the
//           artificial viscosity, advection and RK4 update as above
// FP64 only; the strict namespace keeps the reference's operation order without FMA
// contraction (atan2, sin and cos are CUDA's, within an ulp or two of the C library's).
#include "mf_common.cuh"
#include "mf_kernels.h"

using namespace mfk;
using mfk_host::BodyParams;
using mfk_host::TLArgs;

namespace MF_NS {
namespace {

enum : uint32_t {
	A_ART_VISC = 1u << 6,
	A_ADVECTION = 1u << 11,
	A_DISP = 1u << 12,
	A_GREEN = 1u << 13,
	A_C2N = 1u << 14,
	A_CR_ANISO = 1u << 28,
	A_CR_DISP = 1u << 29,
	A_CR_CAUCHY_GREEN = 1u << 30,
	A_CR_STRESS = 1u << 31,
};

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

__device__ __forceinline__ uint32_t sell_base(const TLArgs& a, uint32_t i) { return a.sl_off[i >> 5] + (i & 31u); }

// a 32-byte per-row record through the read-only path, as two 16-byte loads
__device__ __forceinline__ double4 ld4(const double4* p) {
	const double2* q = reinterpret_cast<const double2*>(p);
	double2 u = __ldg(q), v = __ldg(q + 1);
	return make_double4(u.x, u.y, v.x, v.y);
}

// precomp_sph: W and grad W per listed pair, with the h of particle i
__global__ void k_sph(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                      const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ h, double* w,
                      double* wx, double* wy) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	double xi = x[i], yi = y[i], hi = h[i];
	for (uint32_t q = off[i]; q < off[i + 1]; q++) {
		uint32_t j = nbr[q];
		KR64 k = cubic_spline(xi - x[j], yi - y[j], hi);
		w[q] = k.w;
		wx[q] = k.w_x;
		wy[q] = k.w_y;
	}
}

// the kernel values into the sliced-ELL layout of the gradients
__global__ void k_sell_w(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ sl_off,
                         const double* __restrict__ w, double* sW) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t base = sl_off[i >> 5] + (i & 31u);
	for (uint32_t k = 0; k < off[i + 1] - off[i]; k++) sW[base + 32 * k] = w[off[i] + k];
}

// the reverse pair's gradient per listed pair: entry k of row i (neighbour j) gets the
// gradient at i's place in j's list, zero if j's list does not hold i
__global__ void k_sell_wji(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                           const double* __restrict__ wx, const double* __restrict__ wy,
                           const uint32_t* __restrict__ sl_off, double2* sWji) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t base = sl_off[i >> 5] + (i & 31u);
	for (uint32_t k = 0; k < off[i + 1] - off[i]; k++) {
		uint32_t j = nbr[off[i] + k];
		double2 g = make_double2(0., 0.);
		for (uint32_t q = off[j]; q < off[j + 1]; q++)
			if (nbr[q] == i) {
				g = make_double2(wx[q], wy[q]);
				break;
			}
		sWji[base + 32 * k] = g;
	}
}

// rotation per row: R = [[cos, -sin], [sin, cos]] stored as Rxx, Rxy, Ryx, Ryy
__global__ void __launch_bounds__(256) k_crR(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double* sW = (const double*)a.sW;
	double Xi = a.X[i], Yi = a.Y[i], xi = s.x[i], yi = s.y[i];
	double Axx = 0., Axy = 0., Ayx = 0., Ayy = 0.;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		double w = sW[q];
		double mj = a.m[j];
		double xji = s.x[j] - xi, yji = s.y[j] - yi;
		double Xji = a.X[j] - Xi, Yji = a.Y[j] - Yi;
		Axx += xji * Xji * mj * w;
		Axy += xji * Yji * mj * w;
		Ayx += yji * Xji * mj * w;
		Ayy += yji * Yji * mj * w;
	}
	double x = Axx + Ayy;
	double y = Ayx - Axy;
	double theta = atan2(y, x);
	// R = (cos, -sin; sin, cos) kept as {cos, sin} (Rxy = -sin exactly), with the mass
	// that the pair forces read alongside
	((double4*)a.R)[i] = make_double4(cos(theta), sin(theta), a.m[i], 0.);
}

// the viscosity loop's view of row i: {x, y, vx, vy} and {h, rho, c, m}
__device__ __forceinline__ void write_av(const TLArgs& a, uint32_t i, double c) {
	const mfk_host::StateSoA& s = a.st;
	double4* av = (double4*)a.av;
	av[2 * i] = make_double4(s.x[i], s.y[i], s.vx[i], s.vy[i]);
	av[2 * i + 1] = make_double4(a.h[i], s.rho[i], c, a.m[i]);
}

// displacement gradient in the rotated frame, Cauchy-Green stress, nominal stress
__global__ void __launch_bounds__(256) k_crA(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* sw = (const double2*)a.sw;
	const double4 Ri = ((const double4*)a.R)[i];
	double xi = s.x[i], yi = s.y[i], Xi = a.X[i], Yi = a.Y[i];
	// R^-1 = R^T (derivatives.h:219-222): (cos, sin; -sin, cos)
	double Rixx_inv = Ri.x, Rixy_inv = Ri.y, Riyx_inv = -Ri.y, Riyy_inv = Ri.x;
	double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		double2 w = sw[q];
		double quad_weight = a.qw0[j];
		double xji = s.x[j] - xi, yji = s.y[j] - yi;
		double Xji = a.X[j] - Xi, Yji = a.Y[j] - Yi;
		double uxji = Rixx_inv * xji + Rixy_inv * yji - Xji;
		double uyji = Riyx_inv * xji + Riyy_inv * yji - Yji;
		Hxx += uxji * w.x * quad_weight;
		Hxy += uxji * w.y * quad_weight;
		Hyx += uyji * w.x * quad_weight;
		Hyy += uyji * w.y * quad_weight;
	}
	const BodyParams& pr = a.params[a.body_of[i]];
	// Cauchy-Green: F = I + H (columns (Hxx+1, Hyx), (Hxy, Hyy+1)), E = (F + F^T)/2 - I
	double Sxx = 0., Sxy = 0., Syy = 0.;
	if (a.flags & A_CR_CAUCHY_GREEN) {
		double F00 = Hxx + 1., F01 = Hyx, F10 = Hxy, F11 = Hyy + 1.;
		double E00 = 0.5 * (F00 + F00) - 1.;
		double E01 = 0.5 * (F01 + F10) - 0.;
		double E11 = 0.5 * (F11 + F11) - 1.;
		double D = pr.D, nu = pr.nu;
		Sxx = D * (E00 + nu * E11);
		Syy = D * (E00 * nu + E11);
		Sxy = D * (1 - nu) * E01;
	}
	double Pxx = 0., Pxy = 0., Pyx = 0., Pyy = 0.;
	if (a.flags & A_C2N) cauchy_to_nominal<double>(Hxx, Hxy, Hyx, Hyy, Sxx - 0., Sxy, Syy - 0., Pxx, Pxy, Pyx, Pyy);
	((double4*)a.P)[i] = make_double4(Pxx, Pxy, Pyx, Pyy);
	write_av(a, i, sqrt(pr.K / s.rho[i]));
}

// displacement gradient, Green-St Venant stress and F_e = -2 V (I + H) S per row;
// F_e is stored column-major (F[0][0], F[0][1], F[1][0], F[1][1]) in the P buffer
__global__ void __launch_bounds__(256) k_ptA(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* sw = (const double2*)a.sw;
	const uint32_t flags = a.flags;
	double uxi = s.x[i] - a.X[i], uyi = s.y[i] - a.Y[i];
	double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
	if (flags & A_DISP) {
		uint32_t q = sell_base(a, i), c = a.cnt[i];
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			double2 w = sw[q];
			double qwj = a.qw0[j];
			double uxj = s.x[j] - a.X[j], uyj = s.y[j] - a.Y[j];
			Hxx += (uxj - uxi) * w.x * qwj;
			Hxy += (uxj - uxi) * w.y * qwj;
			Hyx += (uyj - uyi) * w.x * qwj;
			Hyy += (uyj - uyi) * w.y * qwj;
		}
	}
	const BodyParams& pr = a.params[a.body_of[i]];
	double Sxx = s.Sxx[i], Sxy = s.Sxy[i], Syy = s.Syy[i];
	if (flags & A_GREEN) green_stvenant<double>(Hxx, Hxy, Hyx, Hyy, pr.D, pr.nu, Sxx, Sxy, Syy);
	// -2*voli*Ji*Si: the scalar scales J, then the matrix product, k ascending
	double sc = -2 * a.qw0[i];
	double J00 = sc * (Hxx + 1.), J01 = sc * Hyx, J10 = sc * Hxy, J11 = sc * (Hyy + 1.);
	((double4*)a.P)[i] = make_double4(J00 * Sxx + J10 * Sxy, J01 * Sxx + J11 * Sxy, J00 * Sxy + J10 * Syy,
	                                  J01 * Sxy + J11 * Syy);
	write_av(a, i, sqrt(pr.K / s.rho[i]));
}

// pair forces (rotated stresses or elastic potential), contact force, viscosity,
// advection and the RK4 update
template <bool POT>
__global__ void __launch_bounds__(256) k_crB(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* sw = (const double2*)a.sw;
	const double4* P = (const double4*)a.P;
	const double4* R = (const double4*)a.R;
	const double4* av = (const double4*)a.av;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[i]];
	const double rho0 = pr.rho0;
	double vx_t = 0., vy_t = 0.;
	const uint32_t q0 = sell_base(a, i), c = a.cnt[i];
	const double4 Pi = P[i];
	if (POT && (flags & mfk_host::FLAG_POTENTIAL)) {
		const double2* swji = (const double2*)a.sW;
		double mi = a.m[i];
#if !MF_STRICT_FORM
		const double inv_mi = 1. / mi;
#endif
		uint32_t q = q0;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			double2 w = sw[q], wji = swji[q];
			double4 Fj = ld4(P + j);  // F_e column-major: F[0][0], F[0][1], F[1][0], F[1][1]
			double fij0 = Pi.x * w.x + Pi.z * w.y;
			double fij1 = Pi.y * w.x + Pi.w * w.y;
			double fji0 = Fj.x * wji.x + Fj.z * wji.y;
			double fji1 = Fj.y * wji.x + Fj.w * wji.y;
#if MF_STRICT_FORM
			vx_t += 0.5 * (fji0 - fij0) / mi;
			vy_t += 0.5 * (fji1 - fij1) / mi;
#else
			vx_t += 0.5 * (fji0 - fij0) * inv_mi;
			vy_t += 0.5 * (fji1 - fij1) * inv_mi;
#endif
		}
		vx_t += a.fcx[i] / a.m[i];
		vy_t += a.fcy[i] / a.m[i];
	}
	if (!POT && (flags & A_CR_STRESS)) {
		double Pxxi = Pi.x, Pxyi = Pi.y, Pyxi = Pi.z, Pyyi = Pi.w;
		const double4 Ri = R[i];
		double Rxxi = Ri.x, Rxyi = -Ri.y, Ryxi = Ri.y, Ryyi = Ri.x;
		double rhoi21 = 1. / (rho0 * rho0);
		uint32_t q = q0;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			double2 w = sw[q];
			double4 Pj = ld4(P + j);
			double4 Rj = ld4(R + j);  // {cos, sin, m, 0}
			double Rxxj = Rj.x, Rxyj = -Rj.y, Ryxj = Rj.y, Ryyj = Rj.x;
			double mj = Rj.z;
			double rhoj21 = rhoi21;  // 1. / (rho0 * rho0), the same expression per pair
			double aijx = mj * ((Pxxi * rhoi21 + Pj.x * rhoj21) * w.x + (Pxyi * rhoi21 + Pj.y * rhoj21) * w.y);
			double aijy = mj * ((Pyxi * rhoi21 + Pj.z * rhoj21) * w.x + (Pyyi * rhoi21 + Pj.w * rhoj21) * w.y);
			double ajix = -aijx;
			double ajiy = -aijy;
			double aijxprime = aijx * Rxxi + aijy * Rxyi;
			double aijyprime = aijx * Ryxi + aijy * Ryyi;
			double ajixprime = ajix * Rxxj + ajiy * Rxyj;
			double ajiyprime = ajix * Ryxj + ajiy * Ryyj;
			vx_t += 0.5 * (aijxprime - ajixprime);
			vy_t += 0.5 * (aijyprime - ajiyprime);
		}
		vx_t += a.fcx[i] / a.m[i];
		vy_t += a.fcy[i] / a.m[i];
	}
	const double4 ai0 = av[2 * i], ai1 = av[2 * i + 1];
	double xi = ai0.x, yi = ai0.y, vxi = ai0.z, vyi = ai0.w;
	if (flags & A_ART_VISC) {
		double hi = ai1.x, rhoi = ai1.y, ci = ai1.z;
		double alpha = pr.alpha, beta = pr.beta, eta = pr.eta;
		uint32_t q = q0;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			double4 aj0 = ld4(av + 2 * j);
			double vijx = vxi - aj0.z, vijy = vyi - aj0.w;
			double xij = xi - aj0.x, yij = yi - aj0.y;
			double vijposij = vijx * xij + vijy * yij;
			if (vijposij < 0.) {
				double4 aj1 = ld4(av + 2 * j + 1);  // {h, rho, c, m}
				double2 w = sw[q];
				double mj = aj1.w;
				double cij = 0.5 * (ci + aj1.z);
				double hij = 0.5 * (hi + aj1.x);
				double rhoij = 0.5 * (rhoi + aj1.y);
				double r2ij = xij * xij + yij * yij;
				double muij = (hij * vijposij) / (r2ij + eta * eta * hij * hij);
				double piij = (-alpha * cij * muij + beta * muij * muij) / rhoij;
				vx_t += -mj * piij * w.x;
				vy_t += -mj * piij * w.y;
			}
		}
	}
	double d[8];
	d[0] = (flags & A_ADVECTION) ? vxi : 0.;
	d[1] = (flags & A_ADVECTION) ? vyi : 0.;
	d[2] = vx_t;
	d[3] = vy_t;
	d[4] = d[5] = d[6] = d[7] = 0.;  // no density or stress rate in this pipeline
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
			np[q2][i] = bp[q2][i] + d[q2] * dts;
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q2 = 0; q2 < 8; q2++) {
			double v = bp[q2][i] + w6 * (ap[q2][i] + d[q2]);
			bp[q2][i] = v;
			np[q2][i] = v;
		}
		if (!(isfinite(bp[0][i]) && isfinite(bp[1][i]) && isfinite(bp[2][i]) && isfinite(bp[3][i])))
			raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, i);
	}
}

}  // namespace

cudaError_t cr_sph(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* x, const double* y,
                   const double* h, double* w, double* wx, double* wy, cudaStream_t s) {
	k_sph<<<grid1(n, 128), 128, 0, s>>>(n, off, nbr, x, y, h, w, wx, wy);
	return cudaGetLastError();
}

cudaError_t cr_sell_wji(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* wx, const double* wy,
                        const uint32_t* sl_off, void* sWji, cudaStream_t s) {
	k_sell_wji<<<grid1(n, 128), 128, 0, s>>>(n, off, nbr, wx, wy, sl_off, (double2*)sWji);
	return cudaGetLastError();
}

cudaError_t cr_sell_w(uint32_t n, const uint32_t* off, const uint32_t* sl_off, const double* w, double* sW,
                      cudaStream_t s) {
	k_sell_w<<<grid1(n, 128), 128, 0, s>>>(n, off, sl_off, w, sW);
	return cudaGetLastError();
}

namespace {
__global__ void k_cm_pack(TLArgs a);
__global__ void k_cm_R(TLArgs a);
__global__ void k_cm_A(TLArgs a);
template <bool POT>
__global__ void k_cm_B(TLArgs a);
}  // namespace

// part 0: rotation (corotational only), 1: pass A, 2: pass B; mixed form: 10 records,
// 11 rotation, 12 pass A, 13 pass B
cudaError_t cr_stage(const TLArgs& a, int part, cudaStream_t s) {
	unsigned bs = a.block ? a.block : 128;
	const bool pot = (a.flags & mfk_host::FLAG_POTENTIAL) != 0;
	switch (part) {
	case 10: k_cm_pack<<<grid1(a.n_total, 256), 256, 0, s>>>(a); break;
	case 11: k_cm_R<<<grid1(a.n_total, bs), bs, 0, s>>>(a); break;
	case 12: k_cm_A<<<grid1(a.n_total, bs), bs, 0, s>>>(a); break;
	case 13:
		if (pot) k_cm_B<true><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else k_cm_B<false><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		break;
	case 0: k_crR<<<grid1(a.n_total, bs), bs, 0, s>>>(a); break;
	case 1:
		if (pot) k_ptA<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else k_crA<<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		break;
	case 2:
		if (pot) k_crB<true><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		else k_crB<false><<<grid1(a.n_total, bs), bs, 0, s>>>(a);
		break;
	}
	return cudaGetLastError();
}

}  // namespace MF_NS

// ---------------------------------------------------------------------------------
// Mixed form of the corotational and elastic-potential methods: the pair arithmetic and
// the per-row stress (2x2 inversion, Cauchy-Green / Green-St Venant from H) in FP32,
// position differences from float-float records, the RK4 state of x, y, vx, vy in FP64.
// The rotated displacement difference is formed as (R^T - I) X_ji + R^T u_ji, with
// cos - 1 kept as -2 sin^2(theta/2), so that no term cancels in FP32.
namespace MF_NS {
namespace {

__device__ __forceinline__ float ffdiff(float ahi, float alo, float bhi, float blo) {
	return (ahi - bhi) + (alo - blo);
}

// FP64 lists of the set-up -> the mixed form's FP32 per-pair arrays
__global__ void k_cm_lists(uint32_t n, const uint32_t* __restrict__ sl_off, const uint16_t* __restrict__ cnt,
                           const uint32_t* __restrict__ snbr, const double2* __restrict__ sw64,
                           const double* __restrict__ sW64, int potential, const double* __restrict__ X,
                           const double* __restrict__ Y, const double* __restrict__ m, const double* __restrict__ qw,
                           float2* sw, float2* swA, float2* sX, float* sW, float2* swji) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t q = sl_off[i >> 5] + (i & 31u);
	for (uint32_t k = 0; k < cnt[i]; k++, q += 32) {
		uint32_t j = snbr[q];
		double2 w = sw64[q];
		double s = potential ? 1. : m[j];
		sw[q] = make_float2((float)(w.x * s), (float)(w.y * s));
		swA[q] = make_float2((float)(w.x * qw[j]), (float)(w.y * qw[j]));
		if (potential) {
			double2 wr = reinterpret_cast<const double2*>(sW64)[q];
			swji[q] = make_float2((float)wr.x, (float)wr.y);
		} else {
			sX[q] = make_float2((float)(X[j] - X[i]), (float)(Y[j] - Y[i]));
			sW[q] = (float)(m[j] * sW64[q]);
		}
	}
}

// the stage's per-row records from the state (x, y, vx, vy in FP64, rho - rho0 in FP32)
__global__ void k_cm_pack(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const mfk_host::StateSoA& s = a.st;
	const BodyParams& pr = a.params[a.body_of[i]];
	double x = s.x[i], y = s.y[i];
	FF ux = ff_split_bits(x - a.X[i]), uy = ff_split_bits(y - a.Y[i]);
	FF fx = ff_split_bits(x), fy = ff_split_bits(y), fvx = ff_split_bits(s.vx[i]), fvy = ff_split_bits(s.vy[i]);
	((float4*)a.cm_U)[i] = make_float4(ux.hi, ux.lo, uy.hi, uy.lo);
	((float4*)a.cm_X)[i] = make_float4(fx.hi, fx.lo, fy.hi, fy.lo);
	((float4*)a.cm_V)[i] = make_float4(fvx.hi, fvx.lo, fvy.hi, fvy.lo);
	float rho = s.rho_f[i] + pr.frho0;  // the mixed state holds rho - rho0
	((float4*)a.cm_H)[i] = make_float4(((const float*)a.h32)[i], rho, sqrtf(pr.fK / rho), ((const float*)a.m32)[i]);
}

// rotation from the anisotropy tensor, x_ji = X_ji + u_ji
__global__ void __launch_bounds__(256) k_cm_R(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const float4* U = (const float4*)a.cm_U;
	const float2* sX = (const float2*)a.cm_sX;
	const float* sW = (const float*)a.cm_sW;
	const float4 ui = U[i];
	float Axx = 0.f, Axy = 0.f, Ayx = 0.f, Ayy = 0.f;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
#pragma unroll 2
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.snbr[q];
		float2 X2 = sX[q];
		float mW = sW[q];
		float4 uj = __ldg(U + j);
		float xji = X2.x + ffdiff(uj.x, uj.y, ui.x, ui.y);
		float yji = X2.y + ffdiff(uj.z, uj.w, ui.z, ui.w);
		Axx += xji * X2.x * mW;
		Axy += xji * X2.y * mW;
		Ayx += yji * X2.x * mW;
		Ayy += yji * X2.y * mW;
	}
	float th = atan2f(Ayx - Axy, Axx + Ayy);
	float sn, cs;
	sincosf(th, &sn, &cs);
	float h = sinf(0.5f * th);
	((float4*)a.cm_R)[i] = make_float4(cs, sn, -2.f * h * h, ((const float*)a.m32)[i]);
}

// pass A: displacement gradient (rotated, corotational; plain, potential), then per row
// the stress, nominal stress (corotational) or F_e (potential)
__global__ void __launch_bounds__(256) k_cm_A(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const bool pot = (a.flags & mfk_host::FLAG_POTENTIAL) != 0;
	const float4* U = (const float4*)a.cm_U;
	const float2* swA = (const float2*)a.cm_swA;
	const float2* sX = (const float2*)a.cm_sX;
	const float4 ui = U[i];
	float cs = 1.f, sn = 0.f, c1 = 0.f;
	if (!pot) {
		float4 Ri = ((const float4*)a.cm_R)[i];
		cs = Ri.x; sn = Ri.y; c1 = Ri.z;
	}
	float Hxx = 0.f, Hxy = 0.f, Hyx = 0.f, Hyy = 0.f;
	uint32_t q = sell_base(a, i), c = a.cnt[i];
	if (pot ? (a.flags & A_DISP) : (a.flags & A_CR_DISP)) {
#pragma unroll 2
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			float2 w = swA[q];  // gradient times the neighbour's quad weight
			float4 uj = __ldg(U + j);
			float dux = ffdiff(uj.x, uj.y, ui.x, ui.y), duy = ffdiff(uj.z, uj.w, ui.z, ui.w);
			float ux = dux, uy = duy;
			if (!pot) {  // (R^T - I) X_ji + R^T u_ji, R^T = (cos, sin; -sin, cos)
				float2 X2 = sX[q];
				ux = (c1 * X2.x + sn * X2.y) + (cs * dux + sn * duy);
				uy = (-sn * X2.x + c1 * X2.y) + (-sn * dux + cs * duy);
			}
			Hxx += ux * w.x;
			Hxy += ux * w.y;
			Hyx += uy * w.x;
			Hyy += uy * w.y;
		}
	}
	// the per-row part in FP32 (GB300 runs FP64 on a narrow pipe): F = I + H is well
	// conditioned, Green-St Venant takes E from H without forming F^T F - I, and the
	// corotational strain (F + F^T)/2 - I is linear in H
	const BodyParams& pr = a.params[a.body_of[i]];
	const mfk_host::StateSoA& s = a.st;
	float P0 = 0.f, P1 = 0.f, P2 = 0.f, P3 = 0.f;
	if (pot) {
		float Sxx = s.Sxx_f[i], Sxy = s.Sxy_f[i], Syy = s.Syy_f[i];
		if (a.flags & A_GREEN) green_stvenant_h<float>(Hxx, Hxy, Hyx, Hyy, pr.fD, pr.fnu, Sxx, Sxy, Syy);
		float sc = -2.f * ((const float*)a.qw32)[i];
		float J00 = sc * (Hxx + 1.f), J01 = sc * Hyx, J10 = sc * Hxy, J11 = sc * (Hyy + 1.f);
		P0 = J00 * Sxx + J10 * Sxy; P1 = J01 * Sxx + J11 * Sxy;
		P2 = J00 * Sxy + J10 * Syy; P3 = J01 * Sxy + J11 * Syy;
	} else {
		float Sxx = 0.f, Sxy = 0.f, Syy = 0.f;
		if (a.flags & A_CR_CAUCHY_GREEN) {
			float E00 = Hxx, E01 = 0.5f * (Hyx + Hxy), E11 = Hyy;  // (F + F^T)/2 - I
			Sxx = pr.fD * (E00 + pr.fnu * E11);
			Syy = pr.fD * (E00 * pr.fnu + E11);
			Sxy = pr.fD * (1.f - pr.fnu) * E01;
		}
		if (a.flags & A_C2N) cauchy_to_nominal<float>(Hxx, Hxy, Hyx, Hyy, Sxx, Sxy, Syy, P0, P1, P2, P3);
	}
	((float4*)a.cm_P)[i] = make_float4(P0, P1, P2, P3);
}

// pass B: pair forces, contact, viscosity, advection, RK4 (x, y, vx, vy; rho and the
// stresses have no rate in these pipelines)
template <bool POT>
__global__ void __launch_bounds__(256) k_cm_B(TLArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_total) return;
	const float2* sw = (const float2*)a.cm_sw;
	const float4* P = (const float4*)a.cm_P;
	const float4* R = (const float4*)a.cm_R;
	const float4* Xr = (const float4*)a.cm_X;
	const float4* Vr = (const float4*)a.cm_V;
	const float4* Hr = (const float4*)a.cm_H;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[i]];
	const float4 Pi = P[i];
	float fx = 0.f, fy = 0.f;
	const uint32_t q0 = sell_base(a, i), c = a.cnt[i];
	bool forces = false;
	if (POT && (flags & mfk_host::FLAG_POTENTIAL)) {
		forces = true;
		const float2* swji = (const float2*)a.cm_swji;
		uint32_t q = q0;
#pragma unroll 2
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			float2 w = sw[q], wr = swji[q];
			float4 Fj = __ldg(P + j);
			fx += (Fj.x * wr.x + Fj.z * wr.y) - (Pi.x * w.x + Pi.z * w.y);
			fy += (Fj.y * wr.x + Fj.w * wr.y) - (Pi.y * w.x + Pi.w * w.y);
		}
		const float half_mi = 0.5f / ((const float*)a.m32)[i];
		fx *= half_mi;
		fy *= half_mi;
	}
	if (!POT && (flags & A_CR_STRESS)) {
		forces = true;
		const float r21 = (float)(1. / (pr.rho0 * pr.rho0));
		const float4 Ri = R[i];
		uint32_t q = q0;
#pragma unroll 2
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			float2 w = sw[q];  // m_j grad W
			float4 Pj = __ldg(P + j), Rj = __ldg(R + j);
			float ax = ((Pi.x + Pj.x) * w.x + (Pi.y + Pj.y) * w.y) * r21;
			float ay = ((Pi.z + Pj.z) * w.x + (Pi.w + Pj.w) * w.y) * r21;
			// R_i a_ij - R_j a_ji with a_ji = -a_ij, R = (cos, -sin; sin, cos)
			fx += 0.5f * ((ax * Ri.x - ay * Ri.y) + (ax * Rj.x - ay * Rj.y));
			fy += 0.5f * ((ax * Ri.y + ay * Ri.x) + (ax * Rj.y + ay * Rj.x));
		}
	}
	const float4 xi = Xr[i], vi = Vr[i], hi = Hr[i];
	float avx = 0.f, avy = 0.f;
	if (flags & A_ART_VISC) {
		const float alpha = pr.falpha, beta = pr.fbeta, eta2 = pr.feta2;
		uint32_t q = q0;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.snbr[q];
			float4 xj = __ldg(Xr + j), vj = __ldg(Vr + j);
			float xij = ffdiff(xi.x, xi.y, xj.x, xj.y), yij = ffdiff(xi.z, xi.w, xj.z, xj.w);
			float vijx = ffdiff(vi.x, vi.y, vj.x, vj.y), vijy = ffdiff(vi.z, vi.w, vj.z, vj.w);
			float vijposij = vijx * xij + vijy * yij;
			if (vijposij < 0.f) {
				float4 hj = __ldg(Hr + j);  // {h, rho, c, m}
				float2 w = sw[q];
				float mj_w_x = POT ? hj.w * w.x : w.x, mj_w_y = POT ? hj.w * w.y : w.y;  // m_j grad W
				float cij = 0.5f * (hi.z + hj.z), hij = 0.5f * (hi.x + hj.x), rhoij = 0.5f * (hi.y + hj.y);
				float r2ij = xij * xij + yij * yij;
				float muij = __fdividef(hij * vijposij, r2ij + eta2 * hij * hij);
				float piij = __fdividef(-alpha * cij * muij + beta * muij * muij, rhoij);
				avx += -piij * mj_w_x;
				avy += -piij * mj_w_y;
			}
		}
	}
	const mfk_host::StateSoA& s = a.st;
	double d[4];
	d[0] = (flags & A_ADVECTION) ? s.vx[i] : 0.;
	d[1] = (flags & A_ADVECTION) ? s.vy[i] : 0.;
	d[2] = (double)avx;
	d[3] = (double)avy;
	if (forces) {  // the contact term in FP32 (an FP64 division would occupy the narrow FP64 pipe)
		const float inv_m = 1.f / ((const float*)a.m32)[i];
		d[2] += (double)(fx + (float)a.fcx[i] * inv_m);
		d[3] += (double)(fy + (float)a.fcy[i] * inv_m);
	}
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* np[4] = {a.nxt.x, a.nxt.y, a.nxt.vx, a.nxt.vy};
	const uint32_t stg = a.stage;
	const double dt = pr.dt;
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q2 = 0; q2 < 4; q2++) {
			ap[q2][i] = (stg == 0) ? d[q2] : ap[q2][i] + 2 * d[q2];
			np[q2][i] = bp[q2][i] + d[q2] * dts;
		}
		// rho and the stresses carry over unchanged into the next stage's set
		a.nxt.rho_f[i] = a.base.rho_f[i];
		a.nxt.Sxx_f[i] = a.base.Sxx_f[i];
		a.nxt.Sxy_f[i] = a.base.Sxy_f[i];
		a.nxt.Syy_f[i] = a.base.Syy_f[i];
	} else {
		double w6 = dt * 1. / 6.;
		bool ok = true;
#pragma unroll
		for (int q2 = 0; q2 < 4; q2++) {
			double v = bp[q2][i] + w6 * (ap[q2][i] + d[q2]);
			bp[q2][i] = v;
			np[q2][i] = v;
			ok = ok && isfinite(v);
		}
		a.nxt.rho_f[i] = a.base.rho_f[i];
		a.nxt.Sxx_f[i] = a.base.Sxx_f[i];
		a.nxt.Sxy_f[i] = a.base.Sxy_f[i];
		a.nxt.Syy_f[i] = a.base.Syy_f[i];
		if (!ok) raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, i);
	}
}

}  // namespace

cudaError_t cr_mixed_lists(uint32_t n, const uint32_t* sl_off, const uint16_t* cnt, const uint32_t* snbr,
                           const void* sw64, const double* sW64, int potential, const double* X, const double* Y,
                           const double* m, const double* qw, void* sw, void* swA, void* sX, void* sW, void* swji,
                           cudaStream_t s) {
	k_cm_lists<<<(n + 127) / 128, 128, 0, s>>>(n, sl_off, cnt, snbr, (const double2*)sw64, sW64, potential, X, Y, m, qw,
	                                           (float2*)sw, (float2*)swA, (float2*)sX, (float*)sW, (float2*)swji);
	return cudaGetLastError();
}

}  // namespace MF_NS
