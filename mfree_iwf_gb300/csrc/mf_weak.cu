// Weak-form total-Lagrangian kernels with RKPM shape functions (particle_tl_weak;
// tensile_tl_weak, tensile.cpp:731-826; rk4::do_step_weak and step, rk4.h:140-218).
//
// Set-up (once): Gauss points of the quad mesh (gauss_int::update_gauss_points,
// gauss_integration.h:47-123, 2x2 rule), the neighbour lists of Gauss points and of
// particles among the particles (find_neighbors), and the RKPM shape functions of
// both (precomp_rkpm, precomp_shape_functions.h:31-208) in FP64.
//
// Per stage (body.h:60-78 with the action list fused):
//   k_gp_pass   per Gauss point: displacement and velocity gradients from its particle
//               neighbours (derivatives.h:152-200,445-481; a Gauss point itself never
//               moves and has zero velocity, so u_i = v_i = 0 exactly), then L, the
//               continuity rate, EOS, Jaumann rate and P = J F^-1 sigma (cont_mech.h,
//               material.h), and the Gauss point's RK4 update (rho, S).
//   k_p_pass    per particle: the stress divergence that derive_stress_weak_tl
//               (derivatives.h:260-294) *scatters* from Gauss points, here *gathered*
//               over the transposed lists (the Gauss points whose list holds the
//               particle, ascending -- the order in which the scatter adds them), then
//               momentum (cont_mech.h:89-106), advection and the particle's RK4 update.
//   k_smooth    velocity smoothing after the step (correctors.h:171-210).
#include "mf_common.cuh"
#include "mf_kernels.h"
#include "mf_rkpm.cuh"

using namespace mfk;
using mfk_host::BodyParams;
using mfk_host::WeakArgs;

namespace MF_NS {
namespace {

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

enum : uint32_t {
	A_ADVECTION = 1u << 11,
	A_DISP_W = 1u << 19,
	A_VEL_W = 1u << 20,
	A_VGRAD_GP = 1u << 21,
	A_CONT_GP = 1u << 22,
	A_EOS_GP = 1u << 23,
	A_JAUMANN_GP = 1u << 24,
	A_C2N_GP = 1u << 25,
	A_STRESS_W = 1u << 26,
	A_MOMENTUM_W = 1u << 27,
};

// ---------------------------------------------------------------- Gauss points
// update_gauss_points (gauss_integration.h:47-123) for one element of an explicit map
// (ll, lr, tr, tl rows): the Gauss points of the tensor rule of `order` (1 or 2;
// gauss_integration.cpp:38-64), point g = order^2 e + k with k = i order + j in the
// order of get_weight_pos_2d, placed by the nodes' (px, py): their positions (when gx
// is given), the weights J w, and, when fwx is given, the element's shape-function
// gradients (and, with fw, the functions) per (point, node) in node order
// (gauss_integration.h:96-118).  The weak TL set-up runs it once on the reference
// positions; the weak UL form with element maps at every derivative evaluation on the
// stage's positions (body.h:97).
__global__ void k_gauss_quads(uint32_t n_elem, const uint32_t* __restrict__ quads, uint32_t order,
                              const double* __restrict__ px, const double* __restrict__ py, double* gx, double* gy,
                              double* gqw, double* fw, double* fwx, double* fwy, DevStatus* st) {
	uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n_elem) return;
	uint32_t nidx[4] = {quads[4 * e], quads[4 * e + 1], quads[4 * e + 2], quads[4 * e + 3]};
	double mx[4], my[4];
#pragma unroll
	for (int I = 0; I < 4; I++) {
		mx[I] = px[nidx[I]];
		my[I] = py[nidx[I]];
	}
	const double par_x[4] = {-1, +1, +1, -1}, par_y[4] = {-1, -1, +1, +1};
	const double p2[2] = {0.577350269189626, -0.577350269189626};
	const uint32_t npe = order * order;
	for (uint32_t k = 0; k < npe; k++) {
		double xi, eta, local_w;
		if (order == 1) {
			xi = 0.; eta = 0.; local_w = 2. * 2.;
		} else {
			xi = p2[k / 2]; eta = p2[k % 2]; local_w = 1.000000000000000 * 1.000000000000000;
		}
		double N[4];
		const double X1 = -1, Y1 = -1, X2 = 1, Y2 = -1, X3 = 1, Y3 = 1, X4 = -1, Y4 = 1;
		N[0] = 0.25 * (1 + X1 * xi) * (1 + Y1 * eta);
		N[1] = 0.25 * (1 + X2 * xi) * (1 + Y2 * eta);
		N[2] = 0.25 * (1 + X3 * xi) * (1 + Y3 * eta);
		N[3] = 0.25 * (1 + X4 * xi) * (1 + Y4 * eta);
		// transpose(m_node) * N
		double gpx = mx[0] * N[0] + mx[1] * N[1] + mx[2] * N[2] + mx[3] * N[3];
		double gpy = my[0] * N[0] + my[1] * N[1] + my[2] * N[2] + my[3] * N[3];
		// x_xi accumulated element by element as dmat2x2(x_xi11, x_xi21, x_xi12, x_xi22)
		double a00 = 0., a01 = 0., a10 = 0., a11 = 0.;  // column-major [col][row]
#pragma unroll
		for (int I = 0; I < 4; I++) {
			double x_xi11 = 0.25 * mx[I] * par_x[I] * (1 + par_y[I] * eta);
			double x_xi12 = 0.25 * mx[I] * par_y[I] * (1 + par_x[I] * xi);
			double x_xi21 = 0.25 * my[I] * par_x[I] * (1 + par_y[I] * eta);
			double x_xi22 = 0.25 * my[I] * par_y[I] * (1 + par_x[I] * xi);
			a00 = a00 + x_xi11;
			a01 = a01 + x_xi21;
			a10 = a10 + x_xi12;
			a11 = a11 + x_xi22;
		}
		double J = -(a00 * a11 - a10 * a01);
		double w = local_w * J;
		uint32_t g = npe * e + k;
		if (!(w > 0.)) raise(st, ERR_GRID, g);
		if (gx) {
			gx[g] = gpx;
			gy[g] = gpy;
		}
		gqw[g] = w;
		if (fwx) {
			// N_x = N_xi * inverse(x_xi): glm's 2x2 inverse (adjugate times 1/det), then
			// the mat2x4 * mat2x2 product, k ascending
			double inv_det = 1. / (a00 * a11 - a10 * a01);
			double i00 = a11 * inv_det, i01 = -a01 * inv_det, i10 = -a10 * inv_det, i11 = a00 * inv_det;
#pragma unroll
			for (int I = 0; I < 4; I++) {
				double nxi = 0.25 * par_x[I] * (1 + par_y[I] * eta);   // N_xi[0][I]
				double neta = 0.25 * par_y[I] * (1 + par_x[I] * xi);  // N_xi[1][I]
				if (fw) fw[4 * g + I] = N[I];
				fwx[4 * g + I] = nxi * i00 + neta * i01;
				fwy[4 * g + I] = nxi * i10 + neta * i11;
			}
		}
	}
}

__global__ void k_gp_disp(uint32_t n, const double* gx, const double* gy, const double* gX, const double* gY, double* ux,
                          double* uy) {
	uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
	if (g >= n) return;
	ux[g] = gx[g] - gX[g];
	uy[g] = gy[g] - gY[g];
}

// compute_rkpm_correctors + compute_rkpm_shape_function (precomp_shape_functions.h:52-173)
// for query point i over its CSR list of particles; writes w, w_x, w_y per pair.
__global__ void k_rkpm(uint32_t n_to, const double* __restrict__ tx, const double* __restrict__ ty,
                       const double* __restrict__ th, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                       const double* __restrict__ fx, const double* __restrict__ fy, const double* __restrict__ fm,
                       const double* __restrict__ frho, const float* __restrict__ frho_f, double* w_out, double* wx_out,
                       double* wy_out, DevStatus* st) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_to) return;
	auto rho = [&](uint32_t j) { return frho ? frho[j] : (double)frho_f[j]; };
	auto all = [](uint32_t) { return true; };
	auto out = [&](uint32_t q, double w, double wx, double wy) {
		if (w_out) w_out[q] = w;
		if (wx_out) wx_out[q] = wx;
		if (wy_out) wy_out[q] = wy;
	};
	if (!rkpm_row(tx[i], ty[i], th[i], off[i], off[i + 1], nbr, fx, fy, fm, rho, all, out)) raise(st, ERR_SINGULAR, i);
}

// For particle j and the k-th Gauss point i of its transposed list: the position of j
// in i's (ascending) list -- binary search -- gives the pair's gradient.
__global__ void k_transpose_w(uint32_t n_p, const uint32_t* __restrict__ toff, const uint32_t* __restrict__ tnbr,
                              const uint32_t* __restrict__ goff, const uint32_t* __restrict__ gnbr,
                              const double* __restrict__ gwx, const double* __restrict__ gwy, double* twx, double* twy,
                              DevStatus* st) {
	uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= n_p) return;
	for (uint32_t t = toff[j]; t < toff[j + 1]; t++) {
		uint32_t i = tnbr[t];
		uint32_t lo = goff[i], hi = goff[i + 1];
		while (lo < hi) {
			uint32_t mid = (lo + hi) >> 1;
			if (gnbr[mid] < j) lo = mid + 1;
			else hi = mid;
		}
		if (lo < goff[i + 1] && gnbr[lo] == j) {
			twx[t] = gwx[lo];
			twy[t] = gwy[lo];
		} else {
			raise(st, ERR_GRID, j);  // the neighbour relation was not symmetric
			twx[t] = 0.;
			twy[t] = 0.;
		}
	}
}

// CSR -> sliced ELL for the weak lists; values optionally pre-multiplied (mixed form).
__global__ void k_weak_sell(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ nbr,
                            const double* __restrict__ a, const double* __restrict__ b, const uint32_t* __restrict__ sl_off,
                            uint16_t* cnt, uint32_t* snbr, double2* out64, float2* out32,
                            const double* __restrict__ mul_row, const double* __restrict__ mul_nbr) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	uint32_t base = sl_off[i >> 5] + (i & 31u);
	uint32_t q0 = off[i], c = off[i + 1] - q0;
	cnt[i] = (uint16_t)c;
	for (uint32_t k = 0; k < c; k++) {
		uint32_t q = base + 32 * k;
		uint32_t j = nbr[q0 + k];
		snbr[q] = j;
		double va = a ? a[q0 + k] : 0., vb = b ? b[q0 + k] : 0.;
		if (out64) out64[q] = make_double2(va, vb);
		if (out32) {
			double s = (mul_row ? mul_row[i] : 1.) * (mul_nbr ? mul_nbr[j] : 1.);
			out32[q] = make_float2((float)(va * s), (float)(vb * s));
		}
	}
}

__device__ __forceinline__ uint32_t sbase(const uint32_t* sl, uint32_t i) { return sl[i >> 5] + (i & 31u); }

// ------------------------------------------------------------- per stage
__global__ void k_weak_bc(WeakArgs a, int on_base) {
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

// per-Gauss-point part shared by both forms
__device__ __forceinline__ void gp_point(uint32_t flags, const BodyParams& pr, double Hxx, double Hxy, double Hyx,
                                         double Hyy, double Fxx, double Fxy, double Fyx, double Fyy, double rho,
                                         double Sxx, double Sxy, double Syy, double& Pxx, double& Pxy, double& Pyx,
                                         double& Pyy, double& rho_t, double& Sxx_t, double& Sxy_t, double& Syy_t) {
	double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0.;
	if (flags & A_VGRAD_GP) velocity_gradient_tl<double>(Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, vx_x, vx_y, vy_x, vy_y);
	rho_t = 0.;
	if (flags & A_CONT_GP) rho_t = -(rho * (vx_x + vy_y));
	double p = 0.;
	if (flags & A_EOS_GP) p = pr.c0sq * (rho - pr.rho0);
	Sxx_t = Sxy_t = Syy_t = 0.;
	if (flags & A_JAUMANN_GP) jaumann<double>(vx_x, vx_y, vy_x, vy_y, Sxx, Sxy, Syy, pr.G, Sxx_t, Sxy_t, Syy_t);
	Pxx = Pxy = Pyx = Pyy = 0.;
	if (flags & A_C2N_GP) cauchy_to_nominal<double>(Hxx, Hxy, Hyx, Hyy, Sxx - p, Sxy, Syy - p, Pxx, Pxy, Pyx, Pyy);
}

// The per-Gauss-point part of the mixed pass in FP32: GB300 runs FP64 (and every
// conversion from it) on a narrow pipe, and in FP64 this part bounded the pass.  The
// density enters as rho - rho0 (the mixed state), so the EOS takes no cancellation;
// F = I + H and its inverse are well conditioned.
__device__ __forceinline__ void gp_point32(uint32_t flags, const BodyParams& pr, float Hxx, float Hxy, float Hyx,
                                           float Hyy, float Fxx, float Fxy, float Fyx, float Fyy, float drho, float Sxx,
                                           float Sxy, float Syy, float P[4], float e[4]) {
	float vx_x = 0.f, vx_y = 0.f, vy_x = 0.f, vy_y = 0.f;
	if (flags & A_VGRAD_GP) velocity_gradient_tl<float>(Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, vx_x, vx_y, vy_x, vy_y);
	e[0] = 0.f;
	if (flags & A_CONT_GP) e[0] = -((pr.frho0 + drho) * (vx_x + vy_y));
	float p = 0.f;
	if (flags & A_EOS_GP) p = pr.fc0sq * drho;
	e[1] = e[2] = e[3] = 0.f;
	if (flags & A_JAUMANN_GP) jaumann<float>(vx_x, vx_y, vy_x, vy_y, Sxx, Sxy, Syy, pr.fG, e[1], e[2], e[3]);
	P[0] = P[1] = P[2] = P[3] = 0.f;
	if (flags & A_C2N_GP) cauchy_to_nominal<float>(Hxx, Hxy, Hyx, Hyy, Sxx - p, Sxy, Syy - p, P[0], P[1], P[2], P[3]);
}

// The mixed Gauss-point state's RK4 update (rk4.h:154-183) in FP32, the state's own type
__device__ __forceinline__ void gp_rk32(const WeakArgs& a, uint32_t i, float dt, const float e[4], float* gb[4],
                                        float* ga[4], float* gs[4]) {
	const uint32_t stg = a.stage;
	if (stg < 3) {
		const float dts = (stg == 2 ? 1.f : 0.5f) * dt;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ga[q][i] = (stg == 0) ? e[q] : ga[q][i] + 2.f * e[q];
			gs[q][i] = gb[q][i] + e[q] * dts;
		}
	} else {
		const float w6 = dt * (1.f / 6.f);
#pragma unroll
		for (int q = 0; q < 4; q++) {
			float v = gb[q][i] + w6 * (ga[q][i] + e[q]);
			gb[q][i] = v;
			gs[q][i] = v;
		}
	}
}

// Gauss point RK4 update of rho and S (rk4.h:154-183)
template <class T>
__device__ __forceinline__ void gp_rk(const WeakArgs& a, uint32_t i, double dt, const double e[4], T* gb[4], T* ga[4],
                                      T* gs[4]) {
	uint32_t stg = a.stage;
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ga[q][i] = (stg == 0) ? (T)e[q] : (T)(ga[q][i] + (T)2 * (T)e[q]);
			gs[q][i] = (T)(gb[q][i] + (T)e[q] * (T)dts);
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			T v = (T)(gb[q][i] + (T)w6 * (ga[q][i] + (T)e[q]));
			gb[q][i] = v;
			gs[q][i] = v;
		}
	}
}

__global__ void __launch_bounds__(256) k_gp_pass64(WeakArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_g) return;
	const mfk_host::StateSoA& s = a.st;
	const double2* gw = (const double2*)a.g_w;
	uint32_t flags = a.flags;
	// the Gauss point's own displacement x - X (constant: the points do not move; zero
	// unless the set-up moved its body after placing them)
	const double uxi = a.gp_ux[i], uyi = a.gp_uy[i];
	double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0., Fxx = 0., Fxy = 0., Fyx = 0., Fyy = 0.;
	uint32_t q = sbase(a.g_sl, i), c = a.g_cnt[i];
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.g_snbr[q];
		double2 w = gw[q];
		double qwj = a.qw_p[j];
		if (flags & A_DISP_W) {
			double uxj = s.x[j] - a.X[j], uyj = s.y[j] - a.Y[j];
			Hxx += (uxj - uxi) * w.x * qwj;
			Hxy += (uxj - uxi) * w.y * qwj;
			Hyx += (uyj - uyi) * w.x * qwj;
			Hyy += (uyj - uyi) * w.y * qwj;
		}
		if (flags & A_VEL_W) {
			double vxj = s.vx[j], vyj = s.vy[j];
			Fxx += (vxj - 0.) * w.x * qwj;
			Fxy += (vxj - 0.) * w.y * qwj;
			Fyx += (vyj - 0.) * w.x * qwj;
			Fyy += (vyj - 0.) * w.y * qwj;
		}
	}
	const BodyParams& pr = a.params[a.gp_body[i]];
	double* gs[4] = {a.gst.rho, a.gst.Sxx, a.gst.Sxy, a.gst.Syy};
	double* gb[4] = {a.gbase.rho, a.gbase.Sxx, a.gbase.Sxy, a.gbase.Syy};
	double* ga[4] = {a.gacc.rho, a.gacc.Sxx, a.gacc.Sxy, a.gacc.Syy};
	double P[4], e[4];
	gp_point(flags, pr, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, gs[0][i], gs[1][i], gs[2][i], gs[3][i], P[0], P[1], P[2],
	         P[3], e[0], e[1], e[2], e[3]);
	double* gP = (double*)a.gP;
	uint32_t n = a.n_g;
	gP[i] = P[0]; gP[n + i] = P[1]; gP[2 * n + i] = P[2]; gP[3 * n + i] = P[3];
	gp_rk<double>(a, i, pr.dt, e, gb, ga, gs);
}

__global__ void __launch_bounds__(256) k_p_pass64(WeakArgs a) {
	uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= a.n_p) return;
	const double2* tw = (const double2*)a.t_w;
	const double* gP = (const double*)a.gP;
	uint32_t n = a.n_g;
	uint32_t flags = a.flags;
	double vol_node = a.qw_p[j];
	double Pxx_x = 0., Pyx_y = 0., Pxy_x = 0., Pyy_y = 0.;
	if (flags & A_STRESS_W) {
		uint32_t q = sbase(a.t_sl, j), c = a.t_cnt[j];
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t i = a.t_snbr[q];
			double2 w = tw[q];
			double quad_weight = a.gp_qw[i];
			Pxx_x -= gP[i] * w.x * quad_weight * vol_node;
			Pyx_y -= gP[2 * n + i] * w.y * quad_weight * vol_node;
			Pxy_x -= gP[n + i] * w.x * quad_weight * vol_node;
			Pyy_y -= gP[3 * n + i] * w.y * quad_weight * vol_node;
		}
	}
	const mfk_host::StateSoA& s = a.st;
	const BodyParams& pr = a.params[a.body_of[j]];
	double m = a.m[j];
	double d[4];
	d[0] = (flags & A_ADVECTION) ? s.vx[j] : 0.;
	d[1] = (flags & A_ADVECTION) ? s.vy[j] : 0.;
	d[2] = 0.;
	d[3] = 0.;
	if (flags & A_MOMENTUM_W) {
		d[2] += 1. / m * (Pxx_x + Pyx_y) + a.fcx[j] / a.m[j];
		d[3] += 1. / m * (Pxy_x + Pyy_y) + a.fcy[j] / a.m[j];
	}
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* sp[4] = {a.st.x, a.st.y, a.st.vx, a.st.vy};
	uint32_t stg = a.stage;
	double dt = pr.dt;
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ap[q][j] = (stg == 0) ? d[q] : ap[q][j] + 2 * d[q];
			sp[q][j] = bp[q][j] + d[q] * dts;  // own row only: in place
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			double v = bp[q][j] + w6 * (ap[q][j] + d[q]);
			bp[q][j] = v;
			sp[q][j] = v;
		}
		if (!(isfinite(bp[0][j]) && isfinite(bp[1][j]) && isfinite(bp[2][j]) && isfinite(bp[3][j])))
			raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, j);
	}
}

// ---- mixed form: particle displacement and velocity as float-float, FP32 sums
__global__ void k_weak_pack(WeakArgs a) {
	uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= a.n_p) return;
	const mfk_host::StateSoA& s = a.st;
	FF ux = ff_split_bits(s.x[j] - a.X[j]), uy = ff_split_bits(s.y[j] - a.Y[j]);
	FF vx = ff_split_bits(s.vx[j]), vy = ff_split_bits(s.vy[j]);
	float4* pk = (float4*)a.pack;
	pk[2 * j] = make_float4(ux.hi, ux.lo, uy.hi, uy.lo);
	pk[2 * j + 1] = make_float4(vx.hi, vx.lo, vy.hi, vy.lo);
}

__global__ void __launch_bounds__(256, 8) k_gp_pass32(WeakArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_g) return;
	const float2* gw = (const float2*)a.g_w;  // gradient times the particle's quad weight
	const float4* pk = (const float4*)a.pack;
	uint32_t flags = a.flags;
	const FF uxi = ff_split_bits(a.gp_ux[i]), uyi = ff_split_bits(a.gp_uy[i]);
	float Hxx = 0.f, Hxy = 0.f, Hyx = 0.f, Hyy = 0.f, Fxx = 0.f, Fxy = 0.f, Fyx = 0.f, Fyy = 0.f;
	uint32_t q = sbase(a.g_sl, i), c = a.g_cnt[i];
#pragma unroll 2
	for (uint32_t k = 0; k < c; k++, q += 32) {
		uint32_t j = a.g_snbr[q];
		float2 w = gw[q];
		if (flags & A_DISP_W) {
			float4 u = __ldg(pk + 2 * j);
			float ux = (u.x - uxi.hi) + (u.y - uxi.lo), uy = (u.z - uyi.hi) + (u.w - uyi.lo);
			Hxx += ux * w.x;
			Hxy += ux * w.y;
			Hyx += uy * w.x;
			Hyy += uy * w.y;
		}
		if (flags & A_VEL_W) {
			float4 v = __ldg(pk + 2 * j + 1);
			float vx = v.x + v.y, vy = v.z + v.w;
			Fxx += vx * w.x;
			Fxy += vx * w.y;
			Fyx += vy * w.x;
			Fyy += vy * w.y;
		}
	}
	const BodyParams& pr = a.params[a.gp_body[i]];
	float* gs[4] = {a.gst.rho_f, a.gst.Sxx_f, a.gst.Sxy_f, a.gst.Syy_f};
	float* gb[4] = {a.gbase.rho_f, a.gbase.Sxx_f, a.gbase.Sxy_f, a.gbase.Syy_f};
	float* ga[4] = {a.gacc.rho_f, a.gacc.Sxx_f, a.gacc.Sxy_f, a.gacc.Syy_f};
	float P[4], e[4];
	// the mixed Gauss-point state holds rho - rho0
	gp_point32(flags, pr, Hxx, Hxy, Hyx, Hyy, Fxx, Fxy, Fyx, Fyy, gs[0][i], gs[1][i], gs[2][i], gs[3][i], P, e);
	((float4*)a.gP)[i] = make_float4(P[0], P[1], P[2], P[3]);
	gp_rk32(a, i, pr.fdt, e, gb, ga, gs);
}

__global__ void __launch_bounds__(256) k_p_pass32(WeakArgs a) {
	uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= a.n_p) return;
	const float2* tw = (const float2*)a.t_w;  // gradient times both quad weights
	const float4* gP = (const float4*)a.gP;
	uint32_t flags = a.flags;
	float Pxx_x = 0.f, Pyx_y = 0.f, Pxy_x = 0.f, Pyy_y = 0.f;
	if (flags & A_STRESS_W) {
		uint32_t q = sbase(a.t_sl, j), c = a.t_cnt[j];
#pragma unroll 2
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t i = a.t_snbr[q];
			float2 w = tw[q];
			float4 P = __ldg(gP + i);
			Pxx_x -= P.x * w.x;
			Pyx_y -= P.z * w.y;
			Pxy_x -= P.y * w.x;
			Pyy_y -= P.w * w.y;
		}
	}
	const mfk_host::StateSoA& s = a.st;
	const BodyParams& pr = a.params[a.body_of[j]];
	double m = a.m[j];
	double d[4];
	d[0] = (flags & A_ADVECTION) ? s.vx[j] : 0.;
	d[1] = (flags & A_ADVECTION) ? s.vy[j] : 0.;
	d[2] = 0.;
	d[3] = 0.;
	if (flags & A_MOMENTUM_W) {  // in FP32: an FP64 division would occupy the narrow FP64 pipe
		const float inv_m = 1.f / (float)m;
		d[2] = (Pxx_x + Pyx_y) * inv_m + (float)a.fcx[j] * inv_m;
		d[3] = (Pxy_x + Pyy_y) * inv_m + (float)a.fcy[j] * inv_m;
	}
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* sp[4] = {a.st.x, a.st.y, a.st.vx, a.st.vy};
	uint32_t stg = a.stage;
	double dt = pr.dt;
	if (stg < 3) {
		double dts = (stg == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ap[q][j] = (stg == 0) ? d[q] : ap[q][j] + 2 * d[q];
			sp[q][j] = bp[q][j] + d[q] * dts;
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			double v = bp[q][j] + w6 * (ap[q][j] + d[q]);
			bp[q][j] = v;
			sp[q][j] = v;
		}
		if (!(isfinite(bp[0][j]) && isfinite(bp[1][j]) && isfinite(bp[2][j]) && isfinite(bp[3][j])))
			raise(reinterpret_cast<DevStatus*>(a.status), ERR_NONFINITE, j);
	}
}

// correctors_smooth_vel (correctors.h:171-210) on the particles: the smoothed velocity
// goes to the stage set (the next step's first stage copy), then back to the particles.
__global__ void k_smooth(WeakArgs a, int mixed) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_p) return;
	uint32_t q = sbase(a.p_sl, i), c = a.p_cnt[i];
	if (!mixed) {
		const double2* pw = (const double2*)a.p_w;  // (w, 0)
		double vsx = 0., vsy = 0.;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.p_snbr[q];
			double w = pw[q].x, qwj = a.qw_p[j];
			vsx += a.base.vx[j] * w * qwj;
			vsy += a.base.vy[j] * w * qwj;
		}
		a.st.vx[i] = vsx;
		a.st.vy[i] = vsy;
	} else {
		const float2* pw = (const float2*)a.p_w;  // (w * qw_j, 0)
		float vsx = 0.f, vsy = 0.f;
		for (uint32_t k = 0; k < c; k++, q += 32) {
			uint32_t j = a.p_snbr[q];
			float w = pw[q].x;
			vsx += (float)a.base.vx[j] * w;
			vsy += (float)a.base.vy[j] * w;
		}
		a.st.vx[i] = vsx;
		a.st.vy[i] = vsy;
	}
}
__global__ void k_smooth_copy(WeakArgs a) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.n_p) return;
	a.base.vx[i] = a.st.vx[i];
	a.base.vy[i] = a.st.vy[i];
}

__global__ void k_weak_time(uint32_t nb, BodyParams* P) {
	uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b < nb) P[b].time += P[b].dt;
}

}  // namespace

cudaError_t weak_gauss_points(uint32_t n_elem, const uint32_t* quads, uint32_t order, const double* px, const double* py,
                              double* gx, double* gy, double* gqw, double* fw, double* fwx, double* fwy, void* status,
                              cudaStream_t s) {
	if (n_elem == 0) return cudaSuccess;
	k_gauss_quads<<<grid1(n_elem, 128), 128, 0, s>>>(n_elem, quads, order, px, py, gx, gy, gqw, fw, fwx, fwy,
	                                                   reinterpret_cast<DevStatus*>(status));
	return cudaGetLastError();
}

cudaError_t weak_gp_disp(uint32_t n, const double* gx, const double* gy, const double* gX, const double* gY, double* ux,
                         double* uy, cudaStream_t s) {
	if (n == 0) return cudaSuccess;
	k_gp_disp<<<grid1(n, 256), 256, 0, s>>>(n, gx, gy, gX, gY, ux, uy);
	return cudaGetLastError();
}

cudaError_t weak_rkpm(uint32_t n_to, const double* tx, const double* ty, const double* th, const uint32_t* off,
                      const uint32_t* nbr, const double* fx, const double* fy, const double* fm, const double* frho,
                      const float* frho_f, double* w, double* wx, double* wy, void* status, cudaStream_t s) {
	k_rkpm<<<grid1(n_to, 128), 128, 0, s>>>(n_to, tx, ty, th, off, nbr, fx, fy, fm, frho, frho_f, w, wx, wy,
	                                         reinterpret_cast<DevStatus*>(status));
	return cudaGetLastError();
}

cudaError_t weak_transpose(uint32_t n_p, const uint32_t* toff, const uint32_t* tnbr, const uint32_t* goff,
                           const uint32_t* gnbr, const double* gwx, const double* gwy, double* twx, double* twy,
                           void* status, cudaStream_t s) {
	k_transpose_w<<<grid1(n_p, 128), 128, 0, s>>>(n_p, toff, tnbr, goff, gnbr, gwx, gwy, twx, twy,
	                                               reinterpret_cast<DevStatus*>(status));
	return cudaGetLastError();
}

cudaError_t weak_sell(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* a, const double* b,
                      const uint32_t* sl_off, uint16_t* cnt, uint32_t* snbr, void* out64, void* out32,
                      const double* mul_row, const double* mul_nbr, cudaStream_t s) {
	k_weak_sell<<<grid1(n, 128), 128, 0, s>>>(n, off, nbr, a, b, sl_off, cnt, snbr, (double2*)out64, (float2*)out32,
	                                           mul_row, mul_nbr);
	return cudaGetLastError();
}

cudaError_t weak_stage(const WeakArgs& a, bool mixed, int part, cudaStream_t s) {
	// 0: BCs on the stage state, 1: pack (mixed), 2: Gauss-point pass, 3: particle pass,
	// 4: BCs on the particles after the step, 5: smoothing, 6: clocks
	unsigned bs = a.block ? a.block : 128;
	switch (part) {
	case 0:
		if (a.n_bc) k_weak_bc<<<grid1(a.n_bc, 128), 128, 0, s>>>(a, 0);
		break;
	case 1:
		if (mixed) k_weak_pack<<<grid1(a.n_p, 256), 256, 0, s>>>(a);
		break;
	case 2:
		if (mixed) k_gp_pass32<<<grid1(a.n_g, bs), bs, 0, s>>>(a);
		else k_gp_pass64<<<grid1(a.n_g, bs), bs, 0, s>>>(a);
		break;
	case 3:
		if (mixed) k_p_pass32<<<grid1(a.n_p, bs), bs, 0, s>>>(a);
		else k_p_pass64<<<grid1(a.n_p, bs), bs, 0, s>>>(a);
		break;
	case 4:
		if (a.n_bc) k_weak_bc<<<grid1(a.n_bc, 128), 128, 0, s>>>(a, 1);
		break;
	case 5:
		k_smooth<<<grid1(a.n_p, 128), 128, 0, s>>>(a, mixed ? 1 : 0);
		k_smooth_copy<<<grid1(a.n_p, 256), 256, 0, s>>>(a);
		break;
	case 6:
		k_weak_time<<<grid1(a.n_bodies, 128), 128, 0, s>>>(a.n_bodies, const_cast<BodyParams*>(a.params));
		break;
	}
	return cudaGetLastError();
}

}  // namespace MF_NS
