// Project-written stand-in for the small part of the GLM vector/matrix API that
// mfree_iwf uses.  GLM itself is a third-party header-only library that the
// reference does not vendor and does not pin (no lockfile or submodule; its
// README claims no dependencies), and it is not installed here.  This header is
// written from the linear algebra and from GLM's documented conventions only:
//
//   * matrices are column-major: m[c] is column c, m[c][r] is row r of it;
//   * tmat2x2(a, b, c, d) takes column 0 = (a, b), column 1 = (c, d);
//   * tmat2x2(s) is s times the identity;
//   * matCxR has C columns and R rows, matCxR * vecC -> vecR;
//   * normalize(v) = v * (1 / sqrt(dot(v, v)));
//   * the 2x2 inverse is the adjugate scaled by the reciprocal determinant.
//
// It exists only so that the reference's own translation units compile for the
// oracle pin (oracle/_ref).  Last-bit agreement with a genuine GLM build is not
// claimed: this header defines the arithmetic the pinned oracle uses.  It is test
// infrastructure and never part of the product.
#ifndef MF_GLM_SUBSET_HPP
#define MF_GLM_SUBSET_HPP

#include <cmath>
#include <cstddef>

namespace glm {

template <typename T> struct tvec2 {
	T x, y;
	tvec2() : x(0), y(0) {}
	explicit tvec2(T s) : x(s), y(s) {}
	tvec2(T a, T b) : x(a), y(b) {}
	template <typename U> explicit tvec2(const tvec2<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
	T& operator[](std::size_t i) { return i == 0 ? x : y; }
	const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
};

template <typename T> struct tvec3 {
	T x, y, z;
	tvec3() : x(0), y(0), z(0) {}
	explicit tvec3(T s) : x(s), y(s), z(s) {}
	tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
	T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
	const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T> struct tvec4 {
	T x, y, z, w;
	tvec4() : x(0), y(0), z(0), w(0) {}
	explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
	tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
	T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
	const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

// vector arithmetic (component-wise)
template <typename T> tvec2<T> operator+(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x + b.x, a.y + b.y); }
template <typename T> tvec2<T> operator-(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x - b.x, a.y - b.y); }
template <typename T> tvec2<T> operator-(const tvec2<T>& a) { return tvec2<T>(-a.x, -a.y); }
template <typename T> tvec2<T> operator*(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x * b.x, a.y * b.y); }
template <typename T> tvec2<T> operator*(T s, const tvec2<T>& a) { return tvec2<T>(s * a.x, s * a.y); }
template <typename T> tvec2<T> operator*(const tvec2<T>& a, T s) { return tvec2<T>(a.x * s, a.y * s); }
template <typename T> tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <typename T> tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }

template <typename T> T dot(const tvec2<T>& a, const tvec2<T>& b) { tvec2<T> t = a * b; return t.x + t.y; }
template <typename T> tvec2<T> normalize(const tvec2<T>& v) { return v * (static_cast<T>(1) / std::sqrt(dot(v, v))); }

// C columns of R-row vectors
template <typename T> struct tmat2x2 {
	tvec2<T> c[2];
	tmat2x2() { c[0] = tvec2<T>(1, 0); c[1] = tvec2<T>(0, 1); }
	explicit tmat2x2(T s) { c[0] = tvec2<T>(s, 0); c[1] = tvec2<T>(0, s); }
	explicit tmat2x2(int s) { c[0] = tvec2<T>(static_cast<T>(s), 0); c[1] = tvec2<T>(0, static_cast<T>(s)); }
	tmat2x2(T a, T b, T d, T e) { c[0] = tvec2<T>(a, b); c[1] = tvec2<T>(d, e); }
	tmat2x2(const tvec2<T>& a, const tvec2<T>& b) { c[0] = a; c[1] = b; }
	template <typename U> tmat2x2(const tvec2<U>& a, const tvec2<U>& b) { c[0] = tvec2<T>(a); c[1] = tvec2<T>(b); }
	template <typename U> tmat2x2(const tmat2x2<U>& o) { c[0] = tvec2<T>(o[0]); c[1] = tvec2<T>(o[1]); }
	tvec2<T>& operator[](std::size_t i) { return c[i]; }
	const tvec2<T>& operator[](std::size_t i) const { return c[i]; }
	tmat2x2& operator+=(const tmat2x2& o) { c[0] = c[0] + o.c[0]; c[1] = c[1] + o.c[1]; return *this; }
};

template <typename T> struct tmat3x3 {
	tvec3<T> c[3];
	tmat3x3() { c[0] = tvec3<T>(1, 0, 0); c[1] = tvec3<T>(0, 1, 0); c[2] = tvec3<T>(0, 0, 1); }
	explicit tmat3x3(T s) { c[0] = tvec3<T>(s, 0, 0); c[1] = tvec3<T>(0, s, 0); c[2] = tvec3<T>(0, 0, s); }
	tvec3<T>& operator[](std::size_t i) { return c[i]; }
	const tvec3<T>& operator[](std::size_t i) const { return c[i]; }
};

template <typename T> struct tmat2x4 {  // 2 columns, 4 rows
	tvec4<T> c[2];
	tmat2x4() {}
	tvec4<T>& operator[](std::size_t i) { return c[i]; }
	const tvec4<T>& operator[](std::size_t i) const { return c[i]; }
};

template <typename T> struct tmat4x2 {  // 4 columns, 2 rows
	tvec2<T> c[4];
	tmat4x2() {}
	tvec2<T>& operator[](std::size_t i) { return c[i]; }
	const tvec2<T>& operator[](std::size_t i) const { return c[i]; }
};

// element-wise matrix arithmetic
template <typename T> tmat2x2<T> operator+(const tmat2x2<T>& a, const tmat2x2<T>& b) { return tmat2x2<T>(a[0] + b[0], a[1] + b[1]); }
template <typename T> tmat2x2<T> operator-(const tmat2x2<T>& a, const tmat2x2<T>& b) { return tmat2x2<T>(a[0] - b[0], a[1] - b[1]); }
template <typename T> tmat2x2<T> operator*(T s, const tmat2x2<T>& a) { return tmat2x2<T>(s * a[0], s * a[1]); }
template <typename T> tmat2x2<T> operator*(const tmat2x2<T>& a, T s) { return tmat2x2<T>(a[0] * s, a[1] * s); }
inline tmat2x2<double> operator*(int s, const tmat2x2<double>& a) { return static_cast<double>(s) * a; }
template <typename T> tmat3x3<T> operator-(const tmat3x3<T>& a) {
	tmat3x3<T> r;
	for (int col = 0; col < 3; col++) r[col] = -a[col];
	return r;
}

// matrix products: (A*B)[c][r] = sum_k A[k][r] * B[c][k], k ascending
template <typename T> tmat2x2<T> operator*(const tmat2x2<T>& a, const tmat2x2<T>& b) {
	tmat2x2<T> r;
	for (int col = 0; col < 2; col++)
		for (int row = 0; row < 2; row++)
			r[col][row] = a[0][row] * b[col][0] + a[1][row] * b[col][1];
	return r;
}
template <typename T> tvec2<T> operator*(const tmat2x2<T>& m, const tvec2<T>& v) {
	return tvec2<T>(m[0][0] * v.x + m[1][0] * v.y, m[0][1] * v.x + m[1][1] * v.y);
}
template <typename T> tvec3<T> operator*(const tmat3x3<T>& m, const tvec3<T>& v) {
	return tvec3<T>(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
	                m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
	                m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}
// mat4x2 (4 columns, 2 rows) * vec4 -> vec2
template <typename T> tvec2<T> operator*(const tmat4x2<T>& m, const tvec4<T>& v) {
	tvec2<T> r;
	for (int row = 0; row < 2; row++)
		r[row] = m[0][row] * v.x + m[1][row] * v.y + m[2][row] * v.z + m[3][row] * v.w;
	return r;
}
// mat2x4 (2 columns, 4 rows) * mat2x2 -> mat2x4
template <typename T> tmat2x4<T> operator*(const tmat2x4<T>& a, const tmat2x2<T>& b) {
	tmat2x4<T> r;
	for (int col = 0; col < 2; col++)
		for (int row = 0; row < 4; row++)
			r[col][row] = a[0][row] * b[col][0] + a[1][row] * b[col][1];
	return r;
}
// float matrix times double vector (used only by an off-path solver); computed in double
inline tvec2<double> operator*(const tmat2x2<float>& m, const tvec2<double>& v) {
	return tvec2<double>((double)m[0][0] * v.x + (double)m[1][0] * v.y, (double)m[0][1] * v.x + (double)m[1][1] * v.y);
}
inline tvec2<double> operator*(const tmat2x2<double>& m, const tvec2<float>& v) {
	return m * tvec2<double>(v);
}

template <typename T> tmat2x2<T> transpose(const tmat2x2<T>& m) { return tmat2x2<T>(m[0][0], m[1][0], m[0][1], m[1][1]); }
template <typename T> tmat4x2<T> transpose(const tmat2x4<T>& m) {
	tmat4x2<T> r;
	for (int col = 0; col < 4; col++) { r[col][0] = m[0][col]; r[col][1] = m[1][col]; }
	return r;
}

template <typename T> T determinant(const tmat2x2<T>& m) { return m[0][0] * m[1][1] - m[1][0] * m[0][1]; }

template <typename T> tmat2x2<T> inverse(const tmat2x2<T>& m) {
	T inv_det = static_cast<T>(1) / (m[0][0] * m[1][1] - m[1][0] * m[0][1]);
	return tmat2x2<T>(m[1][1] * inv_det, -m[0][1] * inv_det, -m[1][0] * inv_det, m[0][0] * inv_det);
}

typedef tvec2<double> dvec2;
typedef tvec3<double> dvec3;
typedef tvec4<double> dvec4;
typedef tmat2x2<double> dmat2x2;
typedef tmat3x3<double> dmat3x3;
typedef tmat2x4<double> dmat2x4;
typedef tmat2x2<float> mat2x2;

}  // namespace glm

#endif
