// Device-side building blocks shared by the time-step kernels: precision traits,
// the cubic-spline kernel and the 2x2 algebra in the reference's operation order,
// the device error word, and ordered-integer encodings for exact min/max.
//
// Every translation unit that includes this header is compiled twice: once with
// --fmad=false (namespace mf_strict: FP64 that never contracts a*b+c into an FMA,
// the parity form) and once with contraction allowed (namespace mf_fast: the FP64
// and mixed-precision production forms).  MF_NS names the namespace.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef MF_STRICT_FORM
#error "MF_STRICT_FORM must be 1 (the FP64 parity form) or 0"
#endif
#ifndef MF_NS
#error "MF_NS must name the kernel namespace (mf_strict or mf_fast)"
#endif

#define MF_DEV __device__ __forceinline__

namespace mfk {

// Device error word bits (sticky; the host reads and clears them after a step).
enum : uint32_t {
	ERR_NBH_OVERFLOW = 1u << 0,   // neighbour count >= capacity (grid.h:167, neighbor_search.h:142)
	ERR_NO_NEIGHBOR = 1u << 1,    // a particle with no neighbour (grid.h:168)
	ERR_GRID = 1u << 2,           // num_cell >= n (grid.h:114) or a hash outside the grid
	ERR_NONFINITE = 1u << 3,      // NaN/Inf in the state (the reference traps FE_INVALID/FE_OVERFLOW)
	ERR_SINGULAR = 1u << 4,       // a singular corrector or moment matrix (precomp_shape_functions.h:45)
	ERR_CONTACT = 1u << 5,        // an empty master boundary
};

struct DevStatus {
	uint32_t flags;
	uint32_t first_index;  // first particle (global row) that raised a flag
};

MF_DEV void raise(DevStatus* st, uint32_t bit, uint32_t row) {
	uint32_t old = atomicOr(&st->flags, bit);
	if (!(old & bit)) atomicMin(&st->first_index, row);
}

// M_1_PI of the C library, as the reference's kernel.cpp uses it
constexpr double K_1_PI = 0.31830988618379067154;

// 2-D cubic spline (kernel.cpp:20-55), FP64, same operation order.
struct KR64 {
	double w, w_x, w_y;
};
MF_DEV KR64 cubic_spline(double xij, double yij, double h) {
	double h1 = 1. / h;
	double rij = sqrt(xij * xij + yij * yij);
	double fac = 10 * (K_1_PI) / 7.0 * h1 * h1;
	double q = rij * h1;
	KR64 w{0., 0., 0.};
	if (q >= 2.) return w;
	if (q >= 1.) {
		w.w = fac * (0.25 * (2 - q) * (2 - q) * (2 - q));
		if (rij > 1e-12) {
			double der = -0.75 * (2 - q) * (2 - q) * h1 / rij;
			w.w_x = xij * der * fac;
			w.w_y = yij * der * fac;
		}
		return w;
	}
	w.w = fac * (1 - 1.5 * q * q * (1 - 0.5 * q));
	if (rij > 1e-12) {
		double der = -3.0 * q * (1 - 0.75 * q) * h1 / rij;
		w.w_x = xij * der * fac;
		w.w_y = yij * der * fac;
	}
	return w;
}

// The same kernel in FP32 for the mixed-precision form; h1 and fac come in
// precomputed per particle, 1/r through rsqrt.
// float -> double by integer operations, exact: the sign and the 23 mantissa bits move
// across and the exponent is re-biased (127 -> 1023); zeros, infinities and NaNs keep
// their class; a subnormal float's mantissa is normalised (its leading one shifted to
// the implicit bit, the exponent lowered by the shift).  Conversions to and from FP64
// issue on the FP64 pipe, GB300's narrowest, so none is used here.
MF_DEV double f2d(float f) {
	const uint32_t u = __float_as_uint(f);
	const uint32_t e = (u >> 23) & 0xffu;
	uint32_t m = u & 0x7fffffu, e64;
	if (e == 0u) {
		const uint32_t sh = m ? (uint32_t)__clz(m) - 8u : 0u;  // 1..23 for a subnormal
		e64 = m ? 897u - sh : 0u;
		m = (m << sh) & 0x7fffffu;
	} else {
		e64 = e == 255u ? 2047u : e + 896u;
	}
	return __hiloint2double((int)((u & 0x80000000u) | (e64 << 20) | (m >> 3)), (int)(m << 29));
}

// double -> float for a double that holds an FP32 value exactly (an f2d result), by
// integer operations: the exponent re-biased, the mantissa's 23 leading bits kept;
// doubles below FP32's normal range become the FP32 subnormal of the same value.
MF_DEV float d2f_exact(double d) {
	const unsigned long long b = (unsigned long long)__double_as_longlong(d);
	const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
	const uint32_t e = (hi >> 20) & 0x7ffu;
	uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29), e32;
	if (e == 0u) {
		e32 = 0u;
		m = 0u;
	} else if (e == 2047u) {
		e32 = 255u;
	} else if (e >= 897u) {
		e32 = e - 896u;
	} else {  // an FP32 subnormal: the implicit bit shifted into the mantissa
		e32 = 0u;
		m = e > 873u ? (0x800000u | m) >> (897u - e) : 0u;
	}
	return __uint_as_float((hi & 0x80000000u) | (e32 << 23) | m);
}

struct KR32 {
	float w, w_x, w_y;
};
MF_DEV KR32 cubic_spline_f(float xij, float yij, float h1, float fac) {
	float r2 = xij * xij + yij * yij;
	float rinv = rsqrtf(fmaxf(r2, 1e-30f));
	float rij = r2 * rinv;
	float q = rij * h1;
	KR32 w{0.f, 0.f, 0.f};
	if (q >= 2.f) return w;
	float der;
	if (q >= 1.f) {
		float t = 2.f - q;
		w.w = fac * (0.25f * t * t * t);
		der = -0.75f * t * t * h1 * rinv;
	} else {
		w.w = fac * (1.f - 1.5f * q * q * (1.f - 0.5f * q));
		der = -3.0f * q * (1.f - 0.75f * q) * h1 * rinv;
	}
	if (r2 > 1e-24f) {
		w.w_x = xij * der * fac;
		w.w_y = yij * der * fac;
	}
	return w;
}

// Column-major 2x2 matrix: c[col][row], GLM's convention, used to restate the
// reference's glm::dmat2x2 expressions with the same operation order.
template <class T>
struct M2 {
	T c[2][2];
	MF_DEV static M2 make(T a, T b, T d, T e) {  // columns (a,b), (d,e)
		M2 m;
		m.c[0][0] = a; m.c[0][1] = b; m.c[1][0] = d; m.c[1][1] = e;
		return m;
	}
};
template <class T> MF_DEV M2<T> mmul(const M2<T>& a, const M2<T>& b) {
	M2<T> r;
#pragma unroll
	for (int col = 0; col < 2; col++)
#pragma unroll
		for (int row = 0; row < 2; row++) r.c[col][row] = a.c[0][row] * b.c[col][0] + a.c[1][row] * b.c[col][1];
	return r;
}
template <class T> MF_DEV M2<T> mscale(T s, const M2<T>& a) {
	return M2<T>::make(s * a.c[0][0], s * a.c[0][1], s * a.c[1][0], s * a.c[1][1]);
}
template <class T> MF_DEV M2<T> madd(const M2<T>& a, const M2<T>& b) {
	return M2<T>::make(a.c[0][0] + b.c[0][0], a.c[0][1] + b.c[0][1], a.c[1][0] + b.c[1][0], a.c[1][1] + b.c[1][1]);
}
template <class T> MF_DEV M2<T> msub(const M2<T>& a, const M2<T>& b) {
	return M2<T>::make(a.c[0][0] - b.c[0][0], a.c[0][1] - b.c[0][1], a.c[1][0] - b.c[1][0], a.c[1][1] - b.c[1][1]);
}
template <class T> MF_DEV M2<T> mtranspose(const M2<T>& m) { return M2<T>::make(m.c[0][0], m.c[1][0], m.c[0][1], m.c[1][1]); }
template <class T> MF_DEV T mdet(const M2<T>& m) { return m.c[0][0] * m.c[1][1] - m.c[1][0] * m.c[0][1]; }
// adjugate times the reciprocal determinant
template <class T> MF_DEV M2<T> minverse(const M2<T>& m) {
	T inv_det = T(1) / (m.c[0][0] * m.c[1][1] - m.c[1][0] * m.c[0][1]);
	return M2<T>::make(m.c[1][1] * inv_det, -m.c[0][1] * inv_det, -m.c[1][0] * inv_det, m.c[0][0] * inv_det);
}

// Jaumann stress rate (material.h:66-84) in the reference's expression order;
// returns S_t[0][0], S_t[0][1], S_t[1][1].
template <class T>
MF_DEV void jaumann(T vx_x, T vx_y, T vy_x, T vy_y, T Sxx, T Sxy, T Syy, T G, T& dSxx, T& dSxy, T& dSyy) {
	M2<T> epsdot = M2<T>::make(vx_x, T(0.5) * (vx_y + vy_x), T(0.5) * (vx_y + vy_x), vy_y);
	M2<T> omega = M2<T>::make(T(0), T(0.5) * (vy_x - vx_y), T(0.5) * (vx_y - vy_x), T(0));
	M2<T> S = M2<T>::make(Sxx, Sxy, Sxy, Syy);
	M2<T> I = M2<T>::make(T(1), T(0), T(0), T(1));
	T trace_epsdot = epsdot.c[0][0] + epsdot.c[1][1];
	T third_tr = T(1.) / T(3.) * trace_epsdot;
	M2<T> dev = msub(epsdot, mscale(third_tr, I));
	M2<T> S_t = madd(msub(mscale(T(2) * G, dev), mmul(S, omega)), mmul(omega, S));
	dSxx = S_t.c[0][0];
	dSxy = S_t.c[0][1];
	dSyy = S_t.c[1][1];
}

// Cauchy -> nominal stress P = J F^-1 sigma (cont_mech.h:154-169); F from the
// displacement gradient H (column-major F = (Hxx+1, Hyx, Hxy, Hyy+1)).
template <class T>
MF_DEV void cauchy_to_nominal(T Hxx, T Hxy, T Hyx, T Hyy, T sxx, T sxy, T syy, T& Pxx, T& Pxy, T& Pyx, T& Pyy) {
	M2<T> F = M2<T>::make(Hxx + T(1), Hyx, Hxy, Hyy + T(1));
	T J = mdet(F);
	M2<T> sigma = M2<T>::make(sxx, sxy, sxy, syy);
	M2<T> Finv = minverse(F);
	M2<T> P = mmul(mscale(J, Finv), sigma);
	Pxx = P.c[0][0];
	Pxy = P.c[1][0];
	Pyx = P.c[0][1];
	Pyy = P.c[1][1];
}

// Green-St Venant plane-stress law (material.h:132-146)
template <class T>
MF_DEV void green_stvenant(T Hxx, T Hxy, T Hyx, T Hyy, T D, T nu, T& Sxx, T& Sxy, T& Syy) {
	M2<T> F = M2<T>::make(Hxx + T(1), Hyx, Hxy, Hyy + T(1));
	M2<T> C = mmul(mtranspose(F), F);
	M2<T> I = M2<T>::make(T(1), T(0), T(0), T(1));
	M2<T> Esv = mscale(T(0.5), msub(C, I));
	Sxx = D * (Esv.c[0][0] + nu * Esv.c[1][1]);
	Syy = D * (Esv.c[0][0] * nu + Esv.c[1][1]);
	Sxy = D * (T(1) - nu) * Esv.c[1][0];
}

// The same law with E = (F^T F - I) / 2 expanded as (H + H^T + H^T H) / 2 (F = I + H):
// algebraically equal, and free of the cancellation of F^T F - I, which in FP32 would
// leave a relative error of ~1e-7 / |H| in small strains.
template <class T>
MF_DEV void green_stvenant_h(T Hxx, T Hxy, T Hyx, T Hyy, T D, T nu, T& Sxx, T& Sxy, T& Syy) {
	T E00 = Hxx + T(0.5) * (Hxx * Hxx + Hyx * Hyx);
	T E11 = Hyy + T(0.5) * (Hxy * Hxy + Hyy * Hyy);
	T E01 = T(0.5) * (Hxy + Hyx + Hxx * Hxy + Hyx * Hyy);
	Sxx = D * (E00 + nu * E11);
	Syy = D * (E00 * nu + E11);
	Sxy = D * (T(1) - nu) * E01;
}

// L = Fdot F^-1 (cont_mech.h:188-203)
template <class T>
MF_DEV void velocity_gradient_tl(T Hxx, T Hxy, T Hyx, T Hyy, T Fxx, T Fxy, T Fyx, T Fyy, T& vx_x, T& vx_y, T& vy_x, T& vy_y) {
	M2<T> F = M2<T>::make(Hxx + T(1), Hyx, Hxy, Hyy + T(1));
	M2<T> Fdot = M2<T>::make(Fxx, Fyx, Fxy, Fyy);
	M2<T> L = mmul(Fdot, minverse(F));
	vx_x = L.c[0][0];
	vx_y = L.c[1][0];
	vy_x = L.c[0][1];
	vy_y = L.c[1][1];
}

// Order-preserving map of doubles onto uint64 for atomicMin/atomicMax.
MF_DEV unsigned long long ord_encode(double d) {
	unsigned long long u = (unsigned long long)__double_as_longlong(d);
	return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
MF_DEV double ord_decode(unsigned long long u) {
	u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
	return __longlong_as_double((long long)u);
}

// A double split into float hi + float lo: differences of two such values in
// FP32 keep ~1e-7 relative accuracy of the *difference* however large the values.
struct FF {
	float hi, lo;
};
MF_DEV FF ff_split(double d) {
	float hi = (float)d;
	float lo = (float)(d - (double)hi);
	return FF{hi, lo};
}
MF_DEV float ff_diff(FF a, FF b) { return (a.hi - b.hi) + (a.lo - b.lo); }

// The same kind of split from the double's bit pattern, with integer operations only
// (every conversion from FP64 runs on the FP64 pipe, which GB300 keeps narrow): hi is
// the double's leading 24 significant bits (truncated, not rounded), lo the remaining
// 29 bits rounded to FP32, so hi + lo carries ~48 significant bits.  Below 2^-74 lo is
// left zero (its unit would be subnormal in FP32), below 2^-126 hi is a signed zero;
// beyond FP32's range (and inf, nan) hi is the plain conversion.
MF_DEV FF ff_split_bits(double d) {
	const unsigned long long u = (unsigned long long)__double_as_longlong(d);
	const uint32_t h = (uint32_t)(u >> 32), l = (uint32_t)u;
	const uint32_t sign = h & 0x80000000u;
	const int e = (int)((h >> 20) & 0x7ffu);  // biased FP64 exponent
	if (e < 897) return FF{__uint_as_float(sign), 0.f};
	if (e > 1150) return FF{(float)d, 0.f};
	const float hi = __uint_as_float(sign | ((uint32_t)(e - 896) << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
	const uint32_t rest = l & 0x1fffffffu;  // units of 2^(e - 1075)
	const int se = e - 948;                 // biased FP32 exponent of that unit
	float lo = 0.f;
	if (rest != 0u && se > 0) lo = __uint2float_rn(rest) * __uint_as_float((uint32_t)se << 23);
	return FF{hi, sign ? -lo : lo};
}

}  // namespace mfk
