// RKPM shape functions with a linear basis: compute_rkpm_correctors and
// compute_rkpm_shape_function (precomp_shape_functions.h:31-173), in the reference's
// operation order, for one query point over the entries q0, q0 + stride, ... before q1
// of its neighbour list.
// Shared by the weak total-Lagrangian set-up and the per-stage shape functions of the
// weak updated-Lagrangian form.
#pragma once

#include "mf_common.cuh"

// The neighbour volume factor m_j / rho_j of every moment term: the parity form keeps
// the reference's (term * m_j) / rho_j; the fast form multiplies by v_j = m_j / rho_j,
// formed once per neighbour (one FP64 division instead of 27).
#if MF_STRICT_FORM
#define MF_RKPM_VOL * mj / rhoj
#else
#define MF_RKPM_VOL * vj
#endif

namespace MF_NS {
namespace {

// use(q): whether list entry q takes part; rho(j): the neighbour's density;
// out(q, w, w_x, w_y): the shape function and its gradient of entry q.  Returns false
// when the moment matrix is singular (the reference's assert, precomp_shape_functions.h:45).
template <class Rho, class Use, class Out>
__device__ __forceinline__ bool rkpm_row(double xi, double yi, double hi, uint32_t q0, uint32_t q1,
                                         const uint32_t* __restrict__ nbr, const double* __restrict__ fx,
                                         const double* __restrict__ fy, const double* __restrict__ fm, Rho rho, Use use,
                                         Out out, uint32_t stride = 1) {
	bool ok = true;
	double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Mx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
	       My[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // [col][row]
	for (uint32_t q = q0; q != q1; q += stride) {
		if (!use(q)) continue;
		uint32_t j = nbr[q];
		double mj = fm[j], rhoj = rho(j);
#if !MF_STRICT_FORM
		const double vj = mj / rhoj;
#endif
		double xj = fx[j], yj = fy[j];
		double rx = xi - xj, ry = yi - yj;
		const double rx_x = 1., rx_y = 0., ry_x = 0., ry_y = 1.;
		mfk::KR64 w = mfk::cubic_spline(xi - xj, yi - yj, hi);
		M[0][0] += w.w MF_RKPM_VOL;
		M[0][1] += w.w * rx MF_RKPM_VOL;
		M[0][2] += w.w * ry MF_RKPM_VOL;
		M[1][0] += w.w * rx MF_RKPM_VOL;
		M[2][0] += w.w * ry MF_RKPM_VOL;
		M[1][1] += rx * rx * w.w MF_RKPM_VOL;
		M[1][2] += rx * ry * w.w MF_RKPM_VOL;
		M[2][1] += ry * rx * w.w MF_RKPM_VOL;
		M[2][2] += ry * ry * w.w MF_RKPM_VOL;

		Mx[0][0] += w.w_x MF_RKPM_VOL;
		Mx[0][1] += w.w_x * rx MF_RKPM_VOL + w.w * rx_x MF_RKPM_VOL;
		Mx[0][2] += w.w_x * ry MF_RKPM_VOL + w.w * rx_y MF_RKPM_VOL;
		Mx[1][0] += w.w_x * rx MF_RKPM_VOL + w.w * rx_x MF_RKPM_VOL;
		Mx[2][0] += w.w_x * ry MF_RKPM_VOL + w.w * rx_y MF_RKPM_VOL;
		Mx[1][1] += rx * rx * w.w_x MF_RKPM_VOL + w.w * (rx_x * rx + rx * rx_x) MF_RKPM_VOL;
		Mx[1][2] += rx * ry * w.w_x MF_RKPM_VOL + w.w * (rx_x * ry + rx * rx_y) MF_RKPM_VOL;
		Mx[2][1] += rx * ry * w.w_x MF_RKPM_VOL + w.w * (rx_y * rx + ry * rx_x) MF_RKPM_VOL;
		Mx[2][2] += ry * ry * w.w_x MF_RKPM_VOL + w.w * (rx_y * ry + ry * rx_y) MF_RKPM_VOL;

		My[0][0] += w.w_y MF_RKPM_VOL;
		My[0][1] += w.w_y * rx MF_RKPM_VOL + w.w * ry_x MF_RKPM_VOL;
		My[0][2] += w.w_y * ry MF_RKPM_VOL + w.w * ry_y MF_RKPM_VOL;
		My[1][0] += w.w_y * rx MF_RKPM_VOL + w.w * ry_x MF_RKPM_VOL;
		My[2][0] += w.w_y * ry MF_RKPM_VOL + w.w * ry_y MF_RKPM_VOL;
		My[1][1] += rx * rx * w.w_y MF_RKPM_VOL + w.w * (ry_x * rx + rx * ry_x) MF_RKPM_VOL;
		My[1][2] += rx * ry * w.w_y MF_RKPM_VOL + w.w * (ry_x * ry + rx * ry_y) MF_RKPM_VOL;
		My[2][1] += rx * ry * w.w_y MF_RKPM_VOL + w.w * (ry_y * rx + ry * ry_x) MF_RKPM_VOL;
		My[2][2] += ry * ry * w.w_y MF_RKPM_VOL + w.w * (ry_y * ry + ry * ry_y) MF_RKPM_VOL;
	}
	// solve3x3 (Cramer's rule, precomp_shape_functions.h:31-50)
	auto solve = [&](const double r[3], double x[3]) {
		double delta = M[0][0] * M[1][1] * M[2][2] + M[1][0] * M[2][1] * M[0][2] + M[2][0] * M[0][1] * M[1][2] -
		               M[0][2] * M[1][1] * M[2][0] - M[1][2] * M[2][1] * M[0][0] - M[2][2] * M[0][1] * M[1][0];
		double delta_x = r[0] * M[1][1] * M[2][2] + M[1][0] * M[2][1] * r[2] + M[2][0] * r[1] * M[1][2] -
		                 r[2] * M[1][1] * M[2][0] - M[1][2] * M[2][1] * r[0] - M[2][2] * r[1] * M[1][0];
		double delta_y = M[0][0] * r[1] * M[2][2] + r[0] * M[2][1] * M[0][2] + M[2][0] * M[0][1] * r[2] -
		                 M[0][2] * r[1] * M[2][0] - r[2] * M[2][1] * M[0][0] - M[2][2] * M[0][1] * r[0];
		double delta_z = M[0][0] * M[1][1] * r[2] + M[1][0] * r[1] * M[0][2] + r[0] * M[0][1] * M[1][2] -
		                 M[0][2] * M[1][1] * r[0] - M[1][2] * r[1] * M[0][0] - r[2] * M[0][1] * M[1][0];
		if (!(fabs(delta) > 0.)) ok = false;
		x[0] = delta_x / delta;
		x[1] = delta_y / delta;
		x[2] = delta_z / delta;
	};
	double P[3] = {1., 0., 0.}, C[3], Cx[3], Cy[3];
	solve(P, C);
	// rhs = -M_x * C  ((-M_x) * C, column-major product)
	double rx_[3], ry_[3];
#pragma unroll
	for (int r = 0; r < 3; r++) {
		rx_[r] = (-Mx[0][r]) * C[0] + (-Mx[1][r]) * C[1] + (-Mx[2][r]) * C[2];
		ry_[r] = (-My[0][r]) * C[0] + (-My[1][r]) * C[1] + (-My[2][r]) * C[2];
	}
	solve(rx_, Cx);
	solve(ry_, Cy);
	for (uint32_t q = q0; q != q1; q += stride) {
		if (!use(q)) continue;
		uint32_t j = nbr[q];
		double xj = fx[j], yj = fy[j];
		double rx = xi - xj, ry = yi - yj;
		const double rx_x = 1., rx_y = 0., ry_x = 0., ry_y = 1.;
		mfk::KR64 w = mfk::cubic_spline(xi - xj, yi - yj, hi);
		double Corr = (rx * C[1] + ry * C[2]) + C[0];
		double Corr_x = (rx * Cx[1] + ry * Cx[2]) + rx_x * C[1] + rx_y * C[2] + Cx[0];
		double Corr_y = (rx * Cy[1] + ry * Cy[2]) + ry_x * C[1] + ry_y * C[2] + Cy[0];
		out(q, Corr * w.w, Corr_x * w.w + Corr * w.w_x, Corr_y * w.w + Corr * w.w_y);
	}
	return ok;
}

// Float-float arithmetic (an unevaluated sum hi + lo, ~48 significant bits) on the FP32
// pipe, for the mixed form's moment solves: Knuth's TwoSum, Dekker's Fast2Sum and the
// exact product error by one FMA (the error-free steps in explicitly rounded
// operations, so nothing is contracted or reordered).
struct F2 {
	float hi, lo;
};
__device__ __forceinline__ F2 f2_fast(float a, float b) {  // |a| >= |b| (or a = 0)
	const float s = __fadd_rn(a, b);
	return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 f2_add(F2 x, F2 y) {
	const float s = __fadd_rn(x.hi, y.hi);
	const float bb = __fsub_rn(s, x.hi);
	const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
	return f2_fast(s, __fadd_rn(e, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ F2 f2_neg(F2 x) { return F2{-x.hi, -x.lo}; }
__device__ __forceinline__ F2 f2_prod(float a, float b) {  // exact
	const float p = __fmul_rn(a, b);
	return F2{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ F2 f2_mul(float a, F2 y) {
	const float p = __fmul_rn(a, y.hi);
	return f2_fast(p, __fmaf_rn(a, y.lo, __fmaf_rn(a, y.hi, -p)));
}
__device__ __forceinline__ F2 f2_mul(F2 x, F2 y) {
	const float p = __fmul_rn(x.hi, y.hi);
	return f2_fast(p, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.hi, -p))));
}
// 1 / d: the FP32 reciprocal and one Newton step in float-float, r + r (1 - d r)
__device__ __forceinline__ F2 f2_recip(F2 d) {
	const float r = 1.f / d.hi;
	const F2 e = f2_add(F2{1.f, 0.f}, f2_neg(f2_mul(r, d)));
	return f2_add(F2{r, 0.f}, f2_mul(r, e));
}

// The same shape functions for the mixed weak updated-Lagrangian form: the 27 moment
// sums per neighbour in FP32, the three 3x3 solves in float-float (through the
// adjugate), the shape functions in FP32.  The sums run over the offsets scaled by
// 1/h, s = (x_i - x_j)/h, with the gradient scaled by h (d/ds = h d/dx), so that every
// moment entry is of order one: with D = diag(1, 1/h, 1/h) the scaled matrices are M' = D M D and
// M'_x = h D M_x D, their solutions C' = D^-1 C and C'_x = h D^-1 C_x, and
// Corr = C'0 + s.C'(1,2), h Corr_x = s.C'_x(1,2) + C'1 + C'_x0 -- the reference's
// expressions (precomp_shape_functions.h:52-173) in scaled units.  A row is init(h),
// add() per neighbour in ascending slot order, then finish(): each(g) calls g(q, d) for
// the row's neighbours (slot q, FP32 offset d = x_i - x_j) in that order, and out(q, w,
// w_x, w_y) takes the FP32 shape function and its gradient.
struct Rkpm32 {
	float h, ih, fac;
	float M[3][3], Mx[3][3], My[3][3];  // [col][row], scaled; upper triangle

	__device__ __forceinline__ void init(double hi) {
		h = (float)hi;
		ih = 1.f / h;
		fac = (float)(10 * (mfk::K_1_PI) / 7.0) * ih * ih;
#pragma unroll
		for (int a_ = 0; a_ < 3; a_++)
#pragma unroll
			for (int b_ = 0; b_ < 3; b_++) M[a_][b_] = Mx[a_][b_] = My[a_][b_] = 0.f;
	}

	// the moments of one neighbour at offset (rx, ry) = x_i - x_j with volume vj
	__device__ __forceinline__ void add(float rx, float ry, float vj) {
		const mfk::KR32 w = mfk::cubic_spline_f(rx, ry, ih, fac);
		const float sx = rx * ih, sy = ry * ih, gx = w.w_x * h, gy = w.w_y * h;
		const float W = w.w * vj, Gx = gx * vj, Gy = gy * vj;
		M[0][0] += W;            M[0][1] += W * sx;       M[0][2] += W * sy;
		M[1][1] += sx * sx * W;  M[1][2] += sx * sy * W;  M[2][2] += sy * sy * W;
		Mx[0][0] += Gx;
		Mx[0][1] += Gx * sx + W;
		Mx[0][2] += Gx * sy;
		Mx[1][1] += sx * sx * Gx + 2.f * sx * W;
		Mx[1][2] += sx * sy * Gx + sy * W;
		Mx[2][2] += sy * sy * Gx;
		My[0][0] += Gy;
		My[0][1] += Gy * sx;
		My[0][2] += Gy * sy + W;
		My[1][1] += sx * sx * Gy;
		My[1][2] += sx * sy * Gy + sx * W;
		My[2][2] += sy * sy * Gy + 2.f * sy * W;
	}

	// the solves and the shape functions of the neighbours each(f) visits
	template <class Each, class Out>
	__device__ __forceinline__ bool finish(Each each, Out out) const {
		// the three solves through the adjugate of the symmetric moment matrix
		// (A^-1 r = adj(A) r / det A, Cramer's rule with the cofactors shared), in
		// float-float: FP64's accuracy for the solve on the FP32 pipe
		const float a00 = M[0][0], a01 = M[0][1], a02 = M[0][2], a11 = M[1][1], a12 = M[1][2], a22 = M[2][2];
		auto cof = [](float p, float q, float r, float t) {  // p q - r t
			return f2_add(f2_prod(p, q), f2_neg(f2_prod(r, t)));
		};
		const F2 j00 = cof(a11, a22, a12, a12), j01 = cof(a02, a12, a01, a22), j02 = cof(a01, a12, a02, a11);
		const F2 j11 = cof(a00, a22, a02, a02), j12 = cof(a01, a02, a00, a12), j22 = cof(a00, a11, a01, a01);
		const F2 det = f2_add(f2_add(f2_mul(a00, j00), f2_mul(a01, j01)), f2_mul(a02, j02));
		const bool ok = fabsf(det.hi) > 0.f;
		const F2 id = f2_recip(det);
		auto dot3 = [](F2 x0, F2 y0, F2 x1, F2 y1, F2 x2, F2 y2) {
			return f2_add(f2_add(f2_mul(x0, y0), f2_mul(x1, y1)), f2_mul(x2, y2));
		};
		auto solve = [&](const F2 r[3], F2 x[3]) {
			x[0] = f2_mul(dot3(j00, r[0], j01, r[1], j02, r[2]), id);
			x[1] = f2_mul(dot3(j01, r[0], j11, r[1], j12, r[2]), id);
			x[2] = f2_mul(dot3(j02, r[0], j12, r[1], j22, r[2]), id);
		};
		const F2 C[3] = {f2_mul(j00, id), f2_mul(j01, id), f2_mul(j02, id)};  // the solution for P = (1, 0, 0)
		// rx_ = -Ax C, ry_ = -Ay C over the symmetric matrices (stored upper triangle)
		auto sym = [](const float (&X)[3][3], int a_, int b_) { return a_ <= b_ ? X[a_][b_] : X[b_][a_]; };
		F2 rx_[3], ry_[3], Cx[3], Cy[3];
#pragma unroll
		for (int r = 0; r < 3; r++) {
			rx_[r] = f2_neg(f2_add(f2_add(f2_mul(sym(Mx, 0, r), C[0]), f2_mul(sym(Mx, 1, r), C[1])),
			                       f2_mul(sym(Mx, 2, r), C[2])));
			ry_[r] = f2_neg(f2_add(f2_add(f2_mul(sym(My, 0, r), C[0]), f2_mul(sym(My, 1, r), C[1])),
			                       f2_mul(sym(My, 2, r), C[2])));
		}
		solve(rx_, Cx);
		solve(ry_, Cy);
		const float c0 = C[0].hi, c1 = C[1].hi, c2 = C[2].hi;
		const float cx0 = Cx[0].hi, cx1 = Cx[1].hi, cx2 = Cx[2].hi;
		const float cy0 = Cy[0].hi, cy1 = Cy[1].hi, cy2 = Cy[2].hi;
		each([&](uint32_t q, float2 r) {
			const float rx = r.x, ry = r.y;
			const mfk::KR32 w = mfk::cubic_spline_f(rx, ry, ih, fac);
			const float sx = rx * ih, sy = ry * ih;
			const float Corr = (sx * c1 + sy * c2) + c0;
			const float Corr_x = (sx * cx1 + sy * cx2) + c1 + cx0;  // h Corr_x
			const float Corr_y = (sx * cy1 + sy * cy2) + c2 + cy0;  // h Corr_y
			out(q, Corr * w.w, Corr_x * ih * w.w + Corr * w.w_x, Corr_y * ih * w.w + Corr * w.w_y);
		});
		return ok;
	}
};

}  // namespace
}  // namespace MF_NS
