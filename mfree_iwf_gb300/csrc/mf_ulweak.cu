// Weak-form updated-Lagrangian SPH with RKPM shape functions and stress points
// (particle_ul_weak; tensile_ul_weak tensile.cpp:626-729, rotation_ul_weak
// rotation.cpp:466-535, rings_ul_weak_contact rings.cpp:817-934; body.h:80-108,
// rk4.h:140-205).
//
// Set-up (host side): candidate lists of the particles and of the stress points among
// the particles (find_neighbors with distance_manhattan, neighbor_search.h:84-180), and
// per particle the stress points whose candidates hold it, ascending; all sliced by 32
// rows (mfk_host::SlotList).
//
// Per derivative evaluation:
//   k_uw_nbh  (particles, then stress points)  nbh_ellipse (neighbor_ellipse.h:62-127):
//             h and the candidates inside the ellipse, then precomp_rkpm over those
//             (precomp_shape_functions.h:143-208); the mixed form runs k_uw_ff (the
//             stage's float-float positions and FP32 volumes) and k_uw_nbh32 (the
//             ellipse in FP32 within a derived error bound, else FP64; FP32 moments)
//   k_uw_gp   per stress point: integration weight, EOS, velocity gradient
//             (derivatives.h:68-99), Jaumann rate, continuity, interpolated velocity
//             (interpolation.h:32-59) and advection, its stress for the particles,
//             and its RK4 update
//   k_uw_p    per particle: integration weight; the stress divergence that
//             derive_stress_weak_ul (derivatives.h:296-329) scatters from the stress
//             points, gathered over the stress points listing the particle in
//             ascending order (the order the scatter adds them); velocity gradient
//             (derivatives.h:32-66), momentum (cont_mech.h:32-68), continuity,
//             advection, the boundary conditions (body.h:106) and the RK4 update
// After the step: the velocity conditions, then the smoothing of rk4.h:198-204
// (ellipse, weights and shape functions of the particles, correctors.h:171-210).
#include "mf_common.cuh"
#include "mf_kernels.h"
#include "mf_rkpm.cuh"

using namespace mfk;
using mfk_host::BodyParams;
using mfk_host::UWArgs;

namespace MF_NS {
namespace {

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

enum : uint32_t {
	A_RIEMANN = 1u << 1,
	A_DERIVE_VEL = 1u << 5,
	A_CONTINUITY = 1u << 9,
	A_MOMENTUM_UL = 1u << 10,
	A_ADVECTION = 1u << 11,
	A_CONT_GP = 1u << 22,
	A_EOS_GP = 1u << 23,
	A_JAUMANN_GP = 1u << 24,
};

// nbh_ellipse (neighbor_ellipse.h:62-127) of the query point (px, py) over its nq
// candidates in slots q0, q0 + stride, ..., FP64: h = half the farthest candidate's
// distance, mask[q] = 1 for the candidates inside the ellipse; returns their number.
__device__ __forceinline__ uint32_t ellipse64(double px, double py, uint32_t q0, uint32_t nq, uint32_t stride,
                                              const uint32_t* __restrict__ nbr, const double* __restrict__ fx,
                                              const double* __restrict__ fy, double& h_row, uint8_t* mask) {
	const uint32_t q1 = q0 + nq * stride;
	double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0., h = 0.;
	for (uint32_t q = q0; q != q1; q += stride) {
		uint32_t j = nbr[q];
		double dx = px - fx[j], dy = py - fy[j];
		double r2 = dx * dx + dy * dy;
		h = fmax(h, r2);
		Hxx += dx * dx; Hxy += dx * dy;
		Hyx += dy * dx; Hyy += dy * dy;
	}
	h = sqrt(h);
	h /= 2;
	h_row = h;
	// eigen (neighbor_ellipse.h:29-60) of A = (Hxx, Hyx; Hxy, Hyy) / n, columns first
	const double nc = (double)nq;
	const double A00 = Hxx / nc, A01 = Hyx / nc, A10 = Hxy / nc, A11 = Hyy / nc;
	double D0, D1, rax, ray;
	if (fabs(A10) < 1e-9 && fabs(A01) < 1e-9) {
		D0 = A00; D1 = A11; rax = 1.; ray = 0.;
	} else {
		double T = A00 + A11;
		double det = A00 * A11 - A10 * A01;
		double L1 = T / 2 + sqrt(T * T / 4 - det);
		double L2 = T / 2 - sqrt(T * T / 4 - det);
		double l1 = fmin(L1, L2), l2 = fmax(L1, L2);
		D0 = l1; D1 = l2;
		double vx, vy;
		if (fabs(A10) > 1e-12) { vx = l1 - A11; vy = A01; }
		else { vx = A10; vy = l1 - A00; }
		double inv = 1. / sqrt(vx * vx + vy * vy);  // glm::normalize
		rax = vx * inv; ray = vy * inv;
	}
	const double a = 1.6651 * sqrt(D0), b = 1.6651 * sqrt(D1);
#if MF_STRICT_FORM
	const double phi = atan2(ray, rax);
	const double cs = cos(phi), sn = sin(phi);
#else
	// the fast form takes the unit eigenvector itself as (cos phi, sin phi), which the
	// reference's cos(atan2(ray, rax)), sin(...) reproduce to an ulp or two, and
	// multiplies by the reciprocal semi-axes
	const double cs = rax, sn = ray, ia = 1. / a, ib = 1. / b;
#endif
	uint32_t cnt = 0;
	for (uint32_t q = q0; q != q1; q += stride) {
		uint32_t j = nbr[q];
		double xc = fx[j] - px, yc = fy[j] - py;
#if MF_STRICT_FORM
		double left = ((cs * xc + sn * yc) / a);
		double right = ((sn * xc - cs * yc) / b);
#else
		double left = (cs * xc + sn * yc) * ia;
		double right = (sn * xc - cs * yc) * ib;
#endif
		bool in = left * left + right * right <= 1;
		mask[q] = in ? 1 : 0;
		cnt += in ? 1u : 0u;
	}
	return cnt;
}

// nbh_ellipse for query point i over its candidates, then the RKPM shape functions of
// the candidates inside the ellipse (FP64).  With qw_dst the row also stores its
// integration weight for the passes: m / rho (riemann_update_integration_weights) when
// qw_src is null, else qw_src (the weights of the last update).
__global__ void k_uw_nbh(uint32_t n_to, const double* __restrict__ tx, const double* __restrict__ ty,
                         const mfk_host::SlotList cand, const double* __restrict__ fx, const double* __restrict__ fy, const double* __restrict__ fm,
                         const double* __restrict__ frho, double* h_out, uint8_t* mask, double* w, double* wx,
                         double* wy, const double* __restrict__ qw_src, double* qw_dst, DevStatus* st) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_to) return;
	const double px = tx[i], py = ty[i];
	const uint32_t q0 = cand.start[i], nq = cand.cnt[i], S = cand.stride;
	const uint32_t* __restrict__ nbr = cand.nbr;
	double h;
	const uint32_t cnt = ellipse64(px, py, q0, nq, S, nbr, fx, fy, h, mask);
	h_out[i] = h;
	if (cnt == 0) raise(st, ERR_NO_NEIGHBOR, i);
	if (qw_dst) qw_dst[i] = qw_src ? qw_src[i] : fm[i] / frho[i];
	auto rho = [&](uint32_t j) { return frho[j]; };
	auto use = [&](uint32_t q) { return mask[q] != 0; };
	auto out = [&](uint32_t q, double ww, double wwx, double wwy) { w[q] = ww; wx[q] = wwx; wy[q] = wwy; };
	if (!rkpm_row(px, py, h, q0, q0 + nq * S, nbr, fx, fy, fm, rho, use, out, S)) raise(st, ERR_SINGULAR, i);
}

// The mixed form's per-particle inputs of one derivative evaluation: the stage's
// positions and velocities as float-float pairs (x = hi + lo to 48 bits), the FP32
// volumes m / rho, and the particles' integration weights of the evaluation (qw_src, or
// m / rho without it: riemann_update_integration_weights) in FP64 and as a float-float
// pair (qw32: the FP32 rounding, qwlo: the rest).
__global__ void k_uw_ff(uint32_t n, const double* __restrict__ x, const double* __restrict__ y,
                        const double* __restrict__ vx, const double* __restrict__ vy, const double* __restrict__ m,
                        const double* __restrict__ rho, const double* __restrict__ qw_src, double* qw_dst,
                        float4* ff, float4* vff, float* vol, float* qw32, float* qwlo) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const FF px = ff_split_bits(x[i]), py = ff_split_bits(y[i]);
	const FF pvx = ff_split_bits(vx[i]), pvy = ff_split_bits(vy[i]);
	ff[i] = make_float4(px.hi, px.lo, py.hi, py.lo);
	vff[i] = make_float4(pvx.hi, pvx.lo, pvy.hi, pvy.lo);
	vol[i] = (float)m[i] / (float)rho[i];
	const double qw = qw_src ? qw_src[i] : m[i] / rho[i];
	qw_dst[i] = qw;
	const FF w = ff_split(qw);
	qw32[i] = w.hi;
	qwlo[i] = w.lo;
}

// The nq candidates in slots q0, q0 + S, ... in batches of four while cont() holds: a
// batch's list entries and float-float positions are all loaded before f(k, q, j,
// position) runs on any of them, so a thread keeps four gathers in flight.
template <class F, class Cont>
__device__ __forceinline__ void cand4(uint32_t q0, uint32_t nq, uint32_t S, const uint32_t* __restrict__ nbr,
                                      const float4* __restrict__ ff, F f, Cont cont) {
	uint32_t k = 0;
	for (; k + 4 <= nq && cont(); k += 4) {
		uint32_t j[4];
		float4 v[4];
#pragma unroll
		for (int u = 0; u < 4; u++) j[u] = nbr[q0 + (k + u) * S];
#pragma unroll
		for (int u = 0; u < 4; u++) v[u] = ff[j[u]];
#pragma unroll
		for (int u = 0; u < 4; u++) f(k + u, q0 + (k + u) * S, j[u], v[u]);
	}
	for (; k < nq && cont(); k++) {
		const uint32_t q = q0 + k * S, j = nbr[q];
		f(k, q, j, ff[j]);
	}
}

// The mixed form's neighbourhood kernel: the ellipse in FP32 from the float-float
// positions, with the FP64 ellipse (ellipse64) taken over for every row whose FP32
// result could differ from it, so the neighbour sets are the FP64 form's; the RKPM
// moments summed in FP32 during the selection, then the solves (float-float) and the
// shape functions (FP32) of Rkpm32.
//
// Error bound of the FP32 ellipse (first order in u = 2^-24).  An offset x_i - x_j
// from the float-float pairs is within 3u of the exact difference, so a moment sum over
// n candidates is within (n + 7) u of its exact value relative to the sum of its terms'
// magnitudes (|dx dy| <= (dx^2 + dy^2) / 2), and every entry of A = H / n is within
// e = (n + 8) u T of FP64's, T = A00 + A11 (FP64's own error is ~1e-16 relative).
// Axis-aligned (the reference's branch for |A01| < 1e-9): s = x^2 / (k A00) +
// y^2 / (k A11) is within (n + 19) u s.  Otherwise the eigen-decomposition uses the
// discriminant ((A00 - A11)/2)^2 + A01^2 (no cancellation) and the better-conditioned
// of the eigenvector forms (l1 - A11, A01) and (A01, l1 - A00): the smaller eigenvalue
// is within e + 3u T, the larger within e + 3u T relative to T / 2, and the axis
// within 2e / (l2 - l1) + 5u radians, whose effect on s is at most s (l2 - l1) / l1
// per radian; together |s32 - s64| <= (3n + 48) u s T / l1.  The kernel's margin is
// twice the bound: a candidate with |s32 - 1| inside it, an FP64 |A01| within its
// rounding spread of the 1e-9 threshold (summed in FP64 when FP32's is within e of it),
// or a non-finite or near-singular ellipse (T / l1 > 1e4) sends the row to ellipse64.
// h is the FP64 distance of the candidate farthest in FP32 (FP64's h, or one within
// FP32 rounding of it where two candidates tie in FP32).
__global__ void __launch_bounds__(128)
    k_uw_nbh32(uint32_t n_to, const double* __restrict__ tx, const double* __restrict__ ty,
               const mfk_host::SlotList cand, const float4* __restrict__ ff,
               const float* __restrict__ vol, const double* __restrict__ fx, const double* __restrict__ fy,
               const double* __restrict__ fm, const double* __restrict__ frho, double* h_out, uint8_t* mask,
               double* w, double* wx, double* wy, const double* __restrict__ qw_src, double* qw_dst, DevStatus* st) {
	constexpr float U = 5.9604645e-8f;  // 2^-24
	constexpr float K2 = 1.6651f * 1.6651f;
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_to) return;
	const double px = tx[i], py = ty[i];
	const FF qx = ff_split_bits(px), qy = ff_split_bits(py);  // the candidates' split (k_uw_ff)
	const float pxh = qx.hi, pxl = qx.lo, pyh = qy.hi, pyl = qy.lo;
	auto offs = [&](const float4 f) {  // x_i - x_j from j's float-float position
		return make_float2((pxh - f.x) + (pxl - f.y), (pyh - f.z) + (pyl - f.w));
	};
	const uint32_t q0 = cand.start[i], nq = cand.cnt[i], S = cand.stride;
	const uint32_t* __restrict__ nbr = cand.nbr;
	float Hxx = 0.f, Hxy = 0.f, Hyy = 0.f, r2m = -1.f;
	uint32_t jm = 0;  // the candidate farthest in FP32
	cand4(
	    q0, nq, S, nbr, ff,
	    [&](uint32_t, uint32_t, uint32_t j, float4 v) {
		    const float2 d = offs(v);
		    const float r2 = d.x * d.x + d.y * d.y;
		    if (r2 > r2m) { r2m = r2; jm = j; }
		    Hxx += d.x * d.x; Hxy += d.x * d.y; Hyy += d.y * d.y;
	    },
	    [] { return true; });
	const float nf = (float)nq;
	const float A00 = Hxx / nf, A01 = Hxy / nf, A11 = Hyy / nf, T = A00 + A11;
	const float e = (nf + 8.f) * U * T;  // bound on each entry's error
	// the reference's branch: axis-aligned when |A01| < 1e-9.  Where FP32 cannot tell
	// (an absolute threshold: at coarse spacings e exceeds it, and a symmetric
	// neighbourhood has A01 ~ 0), A01 itself is summed in FP64 as the FP64 form sums it;
	// an FP64 A01 closer to the threshold than that sum's own rounding spread (at most
	// (n + 2) 2^-53 T / 2 for n <= ~100 candidates, taken as 1e-14 T) stays undecided.
	const double a01 = fabs((double)A01);
	bool branch = a01 + e < 1e-9 || a01 - e >= 1e-9, axis = a01 < 1e-9;
	if (!branch && T > 0.f) {
		double hxy = 0.;
		for (uint32_t kk = 0, q = q0; kk < nq; kk++, q += S) {
			const uint32_t j = nbr[q];
			const double dx = px - fx[j], dy = py - fy[j];
			hxy += dx * dy;
		}
		const double a01d = fabs(hxy / (double)nq);
		branch = fabs(a01d - 1e-9) > 1e-15 + 1e-14 * (double)T;
		axis = a01d < 1e-9;
	}
	bool sure = T > 0.f && branch;
	float cs, sn, ia2, ib2, bound;
	if (axis) {
		cs = 1.f; sn = 0.f;
		ia2 = 1.f / (K2 * A00); ib2 = 1.f / (K2 * A11);
		bound = nf + 19.f;
		sure = sure && A00 > 0.f && A11 > 0.f;
	} else {
		const float d = 0.5f * (A00 - A11), r = sqrtf(d * d + A01 * A01);
		const float l1 = 0.5f * T - r, l2 = 0.5f * T + r;
		const float vx = d >= 0.f ? A01 : d - r, vy = d >= 0.f ? -(d + r) : A01;
		const float inv = rsqrtf(vx * vx + vy * vy);
		cs = vx * inv; sn = vy * inv;
		ia2 = 1.f / (K2 * l1); ib2 = 1.f / (K2 * l2);
		const float cond = T / l1;
		bound = (3.f * nf + 48.f) * cond;
		sure = sure && l1 > 0.f && cond < 1e4f;
	}
	const float m = 2.f * bound * U;
	const float lo = 1.f - m, hi = 1.f + m;
	double h = 0.;
	if (sure) {
		// FP64's h up to FP32 ties: the FP64 distance of the candidate farthest in FP32
		const double dx = px - fx[jm], dy = py - fy[jm];
		h = sqrt(dx * dx + dy * dy);
		h /= 2;
	}
	// the selection, with the RKPM moments of the selected candidates summed as they
	// are found
	Rkpm32 k;
	k.init(h);
	uint32_t cnt = 0;
	uint64_t bits = 0;  // the selection of the first 64 candidates
	cand4(
	    q0, nq, S, nbr, ff,
	    [&](uint32_t kk, uint32_t q, uint32_t j, float4 v) {
		    const float2 d = offs(v);
		    const float left = cs * d.x + sn * d.y, right = sn * d.x - cs * d.y;
		    const float s = left * left * ia2 + right * right * ib2;
		    sure = sure && (s < lo || s > hi);  // false for NaN
		    const bool in = s <= 1.f;
		    mask[q] = in ? 1 : 0;
		    if (in) {
			    cnt++;
			    if (kk < 64) bits |= 1ull << kk;
			    k.add(d.x, d.y, vol[j]);
		    }
	    },
	    [&] { return sure; });
	// the selected candidates in slot order, g(q, offset): the set bits in batches of
	// four (loads first), then (rows of more than 64 candidates) the stored mask
	auto each = [&](auto g) {
		uint64_t b = bits;
		while (b) {
			uint32_t qs[4], js[4];
			float4 vs[4];
			int nb = 0;
#pragma unroll
			for (int u = 0; u < 4; u++)
				if (b) {
					qs[u] = q0 + (uint32_t)(__ffsll((long long)b) - 1) * S;
					b &= b - 1;
					nb = u + 1;
				}
#pragma unroll
			for (int u = 0; u < 4; u++)
				if (u < nb) js[u] = nbr[qs[u]];
#pragma unroll
			for (int u = 0; u < 4; u++)
				if (u < nb) vs[u] = ff[js[u]];
#pragma unroll
			for (int u = 0; u < 4; u++)
				if (u < nb) g(qs[u], offs(vs[u]));
		}
		for (uint32_t kk = 64; kk < nq; kk++) {
			const uint32_t q = q0 + kk * S;
			if (mask[q]) g(q, offs(ff[nbr[q]]));
		}
	};
	if (!sure) {
		cnt = ellipse64(px, py, q0, nq, S, nbr, fx, fy, h, mask);
		bits = 0;
		for (uint32_t kk = 0; kk < nq && kk < 64; kk++)
			if (mask[q0 + kk * S]) bits |= 1ull << kk;
		k.init(h);
		// the moments in slot order again (each's offsets; the volumes by slot)
		for (uint32_t kk = 0; kk < nq; kk++)
			if (const uint32_t q = q0 + kk * S; mask[q]) {
				const uint32_t j = nbr[q];
				const float2 d = offs(ff[j]);
				k.add(d.x, d.y, vol[j]);
			}
	}
	h_out[i] = h;
	if (cnt == 0) raise(st, ERR_NO_NEIGHBOR, i);
	if (qw_dst) qw_dst[i] = qw_src ? qw_src[i] : fm[i] / frho[i];
	auto out = [&](uint32_t q, float ww, float wwx, float wwy) {
		w[q] = mfk::f2d(ww); wx[q] = mfk::f2d(wwx); wy[q] = mfk::f2d(wwy);
	};
	if (!k.finish(each, out)) raise(st, ERR_SINGULAR, i);
}

// the particles' integration weight of this evaluation (riemann_update_integration_weights),
// stored by k_uw_nbh
__device__ __forceinline__ double p_qw(const UWArgs& a, uint32_t j) { return a.qw_stage[j]; }

// rk_add (rk4.h:52-69) for stages 0-2, the 1-2-2-1 combine (rk4.h:168-182) at stage 3
__device__ __forceinline__ void uw_rk(uint32_t stg, double dt, uint32_t i, int nf, double* const* bp,
                                      double* const* ap, double* const* wp, const double* d) {
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
		for (int q = 0; q < nf; q++) {
			ap[q][i] = (stg == 0) ? d[q] : ap[q][i] + 2 * d[q];
			wp[q][i] = bp[q][i] + d[q] * dts;
		}
	} else {
		double w6 = dt * 1. / 6.;
		for (int q = 0; q < nf; q++) bp[q][i] = bp[q][i] + w6 * (ap[q][i] + d[q]);
	}
}

// The mixed form's sums of k_uw_gp in float-float on the FP32 pipe (the stress points'
// velocity gradient sets their stress rate, so they keep FP64's accuracy): the same
// products and order as the fast FP64 form, from the float-float velocities and
// weights and the FP32 shape functions the mixed neighbourhood kernel stored.
__device__ __forceinline__ void uw_gp_sums_ff(const UWArgs& a, uint32_t i, uint32_t flags, double& vx_x, double& vx_y,
                                              double& vy_x, double& vy_y, double& vxi, double& vyi) {
	F2 lxx{0.f, 0.f}, lxy{0.f, 0.f}, lyx{0.f, 0.f}, lyy{0.f, 0.f}, ix{0.f, 0.f}, iy{0.f, 0.f};
	auto cand = [&](uint8_t in, float4 v, F2 qwj, double gx, double gy, double gw) {
		if (!in) return;
		const F2 vx{v.x, v.y}, vy{v.z, v.w};
		if (flags & mfk_host::FLAG_UW_VEL_WEAK) {
			const F2 tx = f2_mul(d2f_exact(gx), qwj), ty = f2_mul(d2f_exact(gy), qwj);
			lxx = f2_add(lxx, f2_mul(vx, tx)); lxy = f2_add(lxy, f2_mul(vx, ty));
			lyx = f2_add(lyx, f2_mul(vy, tx)); lyy = f2_add(lyy, f2_mul(vy, ty));
		}
		if (flags & mfk_host::FLAG_UW_INTERP) {
			const F2 tw = f2_mul(d2f_exact(gw), qwj);
			ix = f2_add(ix, f2_mul(vx, tw)); iy = f2_add(iy, f2_mul(vy, tw));
		}
	};
	// four candidates' loads (the neighbours' velocities and weights gathered) in flight
	const uint32_t S = a.gc.stride, n = a.gc.cnt[i];
	uint32_t q = a.gc.start[i], k = 0;
	for (; k + 4 <= n; k += 4, q += 4 * S) {
		uint32_t nb[4];
		uint8_t in[4];
		float4 v[4];
		F2 qw[4];
		double gx[4], gy[4], gw[4];
#pragma unroll
		for (int u = 0; u < 4; u++) {
			in[u] = a.gmask[q + u * S];
			nb[u] = a.gc.nbr[q + u * S];
			gx[u] = a.gwx[q + u * S];
			gy[u] = a.gwy[q + u * S];
			gw[u] = a.gw[q + u * S];
		}
#pragma unroll
		for (int u = 0; u < 4; u++) { v[u] = a.vff[nb[u]]; qw[u] = F2{a.qw32[nb[u]], a.qwlo[nb[u]]}; }
#pragma unroll
		for (int u = 0; u < 4; u++) cand(in[u], v[u], qw[u], gx[u], gy[u], gw[u]);
	}
	for (; k < n; k++, q += S) {
		const uint32_t nb = a.gc.nbr[q];
		cand(a.gmask[q], a.vff[nb], F2{a.qw32[nb], a.qwlo[nb]}, a.gwx[q], a.gwy[q], a.gw[q]);
	}
	auto dbl = [](F2 x) { return f2d(x.hi) + f2d(x.lo); };
	vx_x = dbl(lxx); vx_y = dbl(lxy); vy_x = dbl(lyx); vy_y = dbl(lyy); vxi = dbl(ix); vyi = dbl(iy);
}

template <bool MIXED>
__global__ void __launch_bounds__(128) k_uw_gp(UWArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_g) return;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.gbody_of[i]];
	const mfk_host::GSoA& g = a.grd;
	const double rho = g.rho[i];
	const double qw = (flags & mfk_host::FLAG_UW_RIEMANN_GP) ? a.gm[i] / rho : a.gqw_base[i];
	const double p = (flags & A_EOS_GP) ? pr.c0sq * (rho - pr.rho0) : 0.;
	double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0., vxi = 0., vyi = 0.;
	if (MIXED) {
		uw_gp_sums_ff(a, i, flags, vx_x, vx_y, vy_x, vy_y, vxi, vyi);
	} else {
	const uint32_t q1 = a.gc.start[i] + a.gc.cnt[i] * a.gc.stride;
	for (uint32_t q = a.gc.start[i]; q != q1; q += a.gc.stride) {
		if (!a.gmask[q]) continue;
		uint32_t j = a.gc.nbr[q];
		double vxj = a.rd.vx[j], vyj = a.rd.vy[j], qwj = p_qw(a, j);
#if MF_STRICT_FORM
		if (flags & mfk_host::FLAG_UW_VEL_WEAK) {
			vx_x += vxj * a.gwx[q] * qwj;
			vx_y += vxj * a.gwy[q] * qwj;
			vy_x += vyj * a.gwx[q] * qwj;
			vy_y += vyj * a.gwy[q] * qwj;
		}
		if (flags & mfk_host::FLAG_UW_INTERP) {
			vxi += vxj * a.gw[q] * qwj;
			vyi += vyj * a.gw[q] * qwj;
		}
#else
		// the fast form weights each gradient once (w_x q_j), then one FMA per sum
		if (flags & mfk_host::FLAG_UW_VEL_WEAK) {
			const double tx = a.gwx[q] * qwj, ty = a.gwy[q] * qwj;
			vx_x += vxj * tx; vx_y += vxj * ty;
			vy_x += vyj * tx; vy_y += vyj * ty;
		}
		if (flags & mfk_host::FLAG_UW_INTERP) {
			const double tw = a.gw[q] * qwj;
			vxi += vxj * tw; vyi += vyj * tw;
		}
#endif
	}
	}
	const double Sxx = g.Sxx[i], Sxy = g.Sxy[i], Syy = g.Syy[i];
	double d[6] = {0., 0., 0., 0., 0., 0.};  // x_t y_t rho_t Sxx_t Sxy_t Syy_t
	if (flags & A_JAUMANN_GP) jaumann<double>(vx_x, vx_y, vy_x, vy_y, Sxx, Sxy, Syy, pr.G, d[3], d[4], d[5]);
	if (flags & A_CONT_GP) d[2] = 0. - rho * (vx_x + vy_y);
	if (flags & mfk_host::FLAG_UW_ADVECTION_GP) { d[0] = 0. + vxi; d[1] = 0. + vyi; }
	const uint32_t n = a.n_g;
	a.gsig[i] = Sxx - p;
	a.gsig[n + i] = Sxy;
	a.gsig[2 * n + i] = Syy - p;
	a.gsig[3 * n + i] = qw;
	if (a.gsig32) a.gsig32[i] = make_float4((float)(Sxx - p), (float)Sxy, (float)(Syy - p), (float)qw);
	double* bp[6] = {a.gbase.x, a.gbase.y, a.gbase.rho, a.gbase.Sxx, a.gbase.Sxy, a.gbase.Syy};
	double* ap[6] = {a.gacc.x, a.gacc.y, a.gacc.rho, a.gacc.Sxx, a.gacc.Sxy, a.gacc.Syy};
	double* wp[6] = {a.gwr.x, a.gwr.y, a.gwr.rho, a.gwr.Sxx, a.gwr.Sxy, a.gwr.Syy};
	uw_rk(a.stage, pr.dt, i, 6, bp, ap, wp, d);
}

// The mixed form's sums of k_uw_p in FP32: the stress divergence from the stress points'
// FP32 stress and weights (gsig32), the velocity gradient from float-float velocity
// differences; the shape-function gradients are the FP32 values the mixed
// neighbourhood kernel stored (as FP64, read back exactly).  Both feed FP64 rates.
__device__ __forceinline__ void uw_p_sums32(const UWArgs& a, uint32_t j, uint32_t flags, double& Sxx_x, double& Sxy_y,
                                            double& Sxy_x, double& Syy_y, double& vx_x, double& vx_y, double& vy_x,
                                            double& vy_y) {
	const float qwj = a.qw32[j];
	float sxx_x = 0.f, sxy_y = 0.f, sxy_x = 0.f, syy_y = 0.f;
	if (flags & mfk_host::FLAG_UW_STRESS) {
		// one transposed entry: the stress point's FP32 stress and weight (Sxx - p, Sxy,
		// Syy - p, qw) and its gradient at the particle, if the particle is in its ellipse
		auto entry = [&](uint8_t in, float4 g, double gx, double gy) {
			if (!in) return;
			const float c = g.w * qwj, tx = d2f_exact(gx) * c, ty = d2f_exact(gy) * c;
			sxx_x -= g.x * tx; sxy_y -= g.y * ty;
			sxy_x -= g.y * tx; syy_y -= g.z * ty;
		};
		// the entries' loads are scattered over the stress points' slots: four entries'
		// loads are issued before any is used
		const uint32_t S = a.tp.stride, n = a.tp.cnt[j];
		uint32_t t = a.tp.start[j], k = 0;
		for (; k + 4 <= n; k += 4, t += 4 * S) {
			uint32_t q[4], gi[4];
			uint8_t in[4];
			float4 g[4];
			double gx[4], gy[4];
#pragma unroll
			for (int u = 0; u < 4; u++) { q[u] = a.tp_slot[t + u * S]; gi[u] = a.tp.nbr[t + u * S]; }
#pragma unroll
			for (int u = 0; u < 4; u++) {
				in[u] = a.gmask[q[u]];
				g[u] = a.gsig32[gi[u]];
				gx[u] = a.gwx[q[u]];
				gy[u] = a.gwy[q[u]];
			}
#pragma unroll
			for (int u = 0; u < 4; u++) entry(in[u], g[u], gx[u], gy[u]);
		}
		for (; k < n; k++, t += S) {
			const uint32_t q = a.tp_slot[t];
			entry(a.gmask[q], a.gsig32[a.tp.nbr[t]], a.gwx[q], a.gwy[q]);
		}
	}
	float lxx = 0.f, lxy = 0.f, lyx = 0.f, lyy = 0.f;
	if (flags & A_DERIVE_VEL) {
		const float4 vj = a.vff[j];
		auto cand = [&](uint8_t in, float4 vk, float qwk, double gx, double gy) {
			if (!in) return;
			const float tx = d2f_exact(gx) * qwk, ty = d2f_exact(gy) * qwk;
			const float dvx = (vk.x - vj.x) + (vk.y - vj.y), dvy = (vk.z - vj.z) + (vk.w - vj.w);
			lxx += dvx * tx; lxy += dvx * ty;
			lyx += dvy * tx; lyy += dvy * ty;
		};
		// four candidates' loads (the neighbours' velocities and weights gathered) in flight
		const uint32_t S = a.pc.stride, n = a.pc.cnt[j];
		uint32_t q = a.pc.start[j], k = 0;
		for (; k + 4 <= n; k += 4, q += 4 * S) {
			uint32_t nb[4];
			uint8_t in[4];
			float4 vk[4];
			float qw[4];
			double gx[4], gy[4];
#pragma unroll
			for (int u = 0; u < 4; u++) {
				in[u] = a.pmask[q + u * S];
				nb[u] = a.pc.nbr[q + u * S];
				gx[u] = a.pwx[q + u * S];
				gy[u] = a.pwy[q + u * S];
			}
#pragma unroll
			for (int u = 0; u < 4; u++) { vk[u] = a.vff[nb[u]]; qw[u] = a.qw32[nb[u]]; }
#pragma unroll
			for (int u = 0; u < 4; u++) cand(in[u], vk[u], qw[u], gx[u], gy[u]);
		}
		for (; k < n; k++, q += S) {
			const uint32_t nb = a.pc.nbr[q];
			cand(a.pmask[q], a.vff[nb], a.qw32[nb], a.pwx[q], a.pwy[q]);
		}
	}
	Sxx_x = f2d(sxx_x); Sxy_y = f2d(sxy_y); Sxy_x = f2d(sxy_x); Syy_y = f2d(syy_y);
	vx_x = f2d(lxx); vx_y = f2d(lxy); vy_x = f2d(lyx); vy_y = f2d(lyy);
}

template <bool MIXED>
__global__ void __launch_bounds__(128) k_uw_p(UWArgs a) {
	uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= a.n_p) return;
	const uint32_t flags = a.flags;
	const BodyParams& pr = a.params[a.body_of[j]];
	const mfk_host::StateSoA& s = a.rd;
	const double rho = s.rho[j], m = a.m[j], vxj = s.vx[j], vyj = s.vy[j];
	double Sxx_x = 0., Sxy_y = 0., Sxy_x = 0., Syy_y = 0.;
	double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0.;
	if (MIXED) {
		uw_p_sums32(a, j, flags, Sxx_x, Sxy_y, Sxy_x, Syy_y, vx_x, vx_y, vy_x, vy_y);
	} else {
	const double qwj = p_qw(a, j);
	if (flags & mfk_host::FLAG_UW_STRESS) {
		const uint32_t ng = a.n_g;
		const uint32_t t1 = a.tp.start[j] + a.tp.cnt[j] * a.tp.stride;
		for (uint32_t t = a.tp.start[j]; t != t1; t += a.tp.stride) {
			uint32_t q = a.tp_slot[t];
			if (!a.gmask[q]) continue;
			uint32_t gi = a.tp.nbr[t];
			double Sxxi = a.gsig[gi], Sxyi = a.gsig[ng + gi], Syyi = a.gsig[2 * ng + gi], qwi = a.gsig[3 * ng + gi];
#if MF_STRICT_FORM
			Sxx_x -= Sxxi * a.gwx[q] * qwi * qwj;
			Sxy_y -= Sxyi * a.gwy[q] * qwi * qwj;
			Sxy_x -= Sxyi * a.gwx[q] * qwi * qwj;
			Syy_y -= Syyi * a.gwy[q] * qwi * qwj;
#else
			const double c = qwi * qwj, tx = a.gwx[q] * c, ty = a.gwy[q] * c;
			Sxx_x -= Sxxi * tx; Sxy_y -= Sxyi * ty;
			Sxy_x -= Sxyi * tx; Syy_y -= Syyi * ty;
#endif
		}
	}
	if (flags & A_DERIVE_VEL) {
		const uint32_t q1 = a.pc.start[j] + a.pc.cnt[j] * a.pc.stride;
		for (uint32_t q = a.pc.start[j]; q != q1; q += a.pc.stride) {
			if (!a.pmask[q]) continue;
			uint32_t k = a.pc.nbr[q];
			double qwk = p_qw(a, k);
#if MF_STRICT_FORM
			vx_x += (s.vx[k] - vxj) * a.pwx[q] * qwk;
			vx_y += (s.vx[k] - vxj) * a.pwy[q] * qwk;
			vy_x += (s.vy[k] - vyj) * a.pwx[q] * qwk;
			vy_y += (s.vy[k] - vyj) * a.pwy[q] * qwk;
#else
			const double tx = a.pwx[q] * qwk, ty = a.pwy[q] * qwk;
			const double dvx = s.vx[k] - vxj, dvy = s.vy[k] - vyj;
			vx_x += dvx * tx; vx_y += dvx * ty;
			vy_x += dvy * tx; vy_y += dvy * ty;
#endif
		}
	}
	}
	double d[5] = {0., 0., 0., 0., 0.};  // x_t y_t vx_t vy_t rho_t
	if (flags & A_MOMENTUM_UL) {
		d[2] = 0. + (1. / rho * (Sxx_x + Sxy_y) + a.fcx[j] / m);
		d[3] = 0. + (1. / rho * (Sxy_x + Syy_y) + a.fcy[j] / m);
	}
	if (flags & mfk_host::FLAG_UW_MOMENTUM_W) {
		d[2] = d[2] + (1. / m * (Sxx_x + Sxy_y) + a.fcx[j] / m);
		d[3] = d[3] + (1. / m * (Sxy_x + Syy_y) + a.fcy[j] / m);
	}
	if (flags & A_CONTINUITY) d[4] = 0. - rho * (vx_x + vy_y);
	if (flags & A_ADVECTION) { d[0] = 0. + vxj; d[1] = 0. + vyj; }
	uint32_t bc = a.bc_of[j];
	if (bc != ~0u) {  // left/right_bndry_fun_ul after the actions (body.h:106)
		d[0] = a.bc_v[bc];
		d[1] = 0.;
		d[2] = 0.;
		d[3] = 0.;
	}
	double* bp[5] = {a.base.x, a.base.y, a.base.vx, a.base.vy, a.base.rho};
	double* ap[5] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy, a.acc.rho};
	double* wp[5] = {a.wr.x, a.wr.y, a.wr.vx, a.wr.vy, a.wr.rho};
	uw_rk(a.stage, pr.dt, j, 5, bp, ap, wp, d);
	if (a.stage == 3 && !(isfinite(bp[0][j]) && isfinite(bp[1][j]) && isfinite(bp[2][j]) && isfinite(bp[3][j])))
		raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, j);
}

// correctors_smooth_vel (correctors.h:171-210) over the particles' fresh ellipse lists;
// the smoothed velocities go to the accumulator arrays first (every row reads the
// unsmoothed ones), then k_uw_smooth_copy moves them into the state
__global__ void k_uw_smooth(UWArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_p) return;
	double vsx = 0., vsy = 0.;
	const uint32_t q1 = a.pc.start[i] + a.pc.cnt[i] * a.pc.stride;
	for (uint32_t q = a.pc.start[i]; q != q1; q += a.pc.stride) {
		if (!a.pmask[q]) continue;
		uint32_t k = a.pc.nbr[q];
		vsx += a.base.vx[k] * a.pw[q] * a.qw_base[k];
		vsy += a.base.vy[k] * a.pw[q] * a.qw_base[k];
	}
	a.acc.x[i] = vsx;
	a.acc.y[i] = vsy;
}

__global__ void k_uw_smooth_copy(UWArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_p) return;
	a.base.vx[i] = a.acc.x[i];
	a.base.vy[i] = a.acc.y[i];
}

}  // namespace

cudaError_t uw_nbh(uint32_t n_to, const double* tx, const double* ty, const mfk_host::SlotList& cand,
                   const double* fx, const double* fy, const double* fm, const double* frho, double* h_out,
                   uint8_t* mask, double* w, double* wx, double* wy, const double* qw_src, double* qw_dst,
                   const void* ff, const float* vol, void* status, cudaStream_t s) {
	if (n_to == 0) return cudaSuccess;
	if (ff)
		k_uw_nbh32<<<grid1(n_to, 128), 128, 0, s>>>(n_to, tx, ty, cand, reinterpret_cast<const float4*>(ff), vol,
		                                            fx, fy, fm, frho, h_out, mask, w, wx, wy, qw_src, qw_dst,
		                                            reinterpret_cast<DevStatus*>(status));
	else
		k_uw_nbh<<<grid1(n_to, 128), 128, 0, s>>>(n_to, tx, ty, cand, fx, fy, fm, frho, h_out, mask, w, wx, wy,
		                                          qw_src, qw_dst, reinterpret_cast<DevStatus*>(status));
	return cudaGetLastError();
}

cudaError_t uw_ff(uint32_t n, const double* x, const double* y, const double* vx, const double* vy, const double* m,
                  const double* rho, const double* qw_src, double* qw_dst, void* ff, void* vff, float* vol,
                  float* qw32, float* qwlo, cudaStream_t s) {
	if (n == 0) return cudaSuccess;
	k_uw_ff<<<grid1(n, 256), 256, 0, s>>>(n, x, y, vx, vy, m, rho, qw_src, qw_dst, reinterpret_cast<float4*>(ff),
	                                      reinterpret_cast<float4*>(vff), vol, qw32, qwlo);
	return cudaGetLastError();
}

// part 0: stress points, 1: particles, 2: smoothing sums, 3: smoothing copy
cudaError_t uw_stage(const UWArgs& a, int part, cudaStream_t s) {
	const unsigned bs = 128;  // the passes' launch bounds
	switch (part) {
	case 0:
		if (a.n_g && a.vff) k_uw_gp<true><<<grid1(a.n_g, bs), bs, 0, s>>>(a);
		else if (a.n_g) k_uw_gp<false><<<grid1(a.n_g, bs), bs, 0, s>>>(a);
		break;
	case 1:
		if (a.n_p && a.vff) k_uw_p<true><<<grid1(a.n_p, bs), bs, 0, s>>>(a);
		else if (a.n_p) k_uw_p<false><<<grid1(a.n_p, bs), bs, 0, s>>>(a);
		break;
	case 2: if (a.n_p) k_uw_smooth<<<grid1(a.n_p, 128), 128, 0, s>>>(a); break;
	case 3: if (a.n_p) k_uw_smooth_copy<<<grid1(a.n_p, 128), 128, 0, s>>>(a); break;
	}
	return cudaGetLastError();
}

}  // namespace MF_NS
