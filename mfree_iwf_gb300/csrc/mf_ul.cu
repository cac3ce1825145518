// Updated-Lagrangian (Gray-Monaghan) SPH time-step kernels.
//
// One derivative evaluation of the reference (body::compute_time_derivatives for
// particle_ul, body.h:125-148) rebuilds the cell grid, sorts the particles by cell
// hash, builds Verlet lists, evaluates the kernel per pair and runs the action list
// (rings.cpp:86-96).  Here that becomes, per RK4 stage, for all bodies at once:
//
//   ul_bbox      per-body bounding box and h_max        (grid.h:83-104)
//   ul_geom      per-body cell geometry, cell offsets   (grid.h:105-115)
//   ul_hash      global cell key per row                (grid.h:35-41)
//   CUB radix sort of (key, row)                        (body.h:137)
//   ul_cells     cell start table, empty cells filled from the right (grid.h:48-81)
//   ul_gather    the rows' stage state in cell order, with the per-particle actions
//                EOS (material.h:37-64), artificial stress (correctors.h:37-81) and
//                integration weights (riemann_integration.h:28-33) fused in
//   ul_pair      one thread per row: walks the 3x3 cell stencil of the reference grid
//                (grid.h:117-177), evaluates W/gradW (kernel.cpp:20-55) and every pair
//                action at once -- derive_stress_monaghan (derivatives.h:378-443),
//                derive_velocity (:32-66), artificial viscosity (correctors.h:83-137),
//                XSPH (:139-169) -- then the per-particle actions Jaumann rate
//                (material.h:66-100), continuity, momentum and advection
//                (cont_mech.h:32-49,108-142) and the RK4 update (rk4.h:52-108).
//
// Neighbour lists are never stored: the pair kernel re-derives them from the cell
// table with the reference's predicate r^2 <= 4 h_i^2 + eps, evaluated without FMA
// contraction so the neighbour sets are the reference's, bit for bit.
#include <cub/device/device_radix_sort.cuh>

#include "mf_common.cuh"
#include "mf_kernels.h"

using namespace mfk;
using mfk_host::BodyParams;
using mfk_host::Geom;
using mfk_host::ULArgs;

namespace MF_NS {
namespace {

enum : uint32_t {
	A_RIEMANN = 1u << 1,
	A_EOS = 1u << 2,
	A_ART_STRESS = 1u << 3,
	A_STRESS_MGHN = 1u << 4,
	A_DERIVE_VEL = 1u << 5,
	A_ART_VISC = 1u << 6,
	A_XSPH = 1u << 7,
	A_JAUMANN = 1u << 8,
	A_CONTINUITY = 1u << 9,
	A_MOMENTUM_UL = 1u << 10,
	A_ADVECTION = 1u << 11,
	A_GOD_CONT = mfk_host::FLAG_GODUNOV_CONTINUITY,
	A_GOD_MOM = mfk_host::FLAG_GODUNOV_MOMENTUM,
};

// Cell-ordered record of one particle's stage state plus per-particle derived
// quantities.  FP64 form: 16 doubles = 128 bytes, loaded as 8 x 16 B.  With the
// Godunov actions (which exclude the artificial stress) Rxx holds the pressure p and
// Rxy the stress Syy itself.
struct __align__(16) Rec64 {
	double x, y, vx, vy;
	double m, h, rho, sxx;   // sxx = Sxx - p
	double sxy, syy, Rxx, Rxy;
	double Ryy, c, qw, rho21;  // c = sqrt(K/rho), qw = m/rho (or the stored weight), rho21 = 1/rho^2
};
// Mixed form: positions and velocities as float-float, the rest FP32: 80 bytes.
struct __align__(16) Rec32 {
	FF x, y, vx, vy;
	float m, h, rho, sxx;
	float sxy, syy, Rxx, Rxy;
	float Ryy, c, qw, rho21;
};

__device__ __forceinline__ Rec64 load_rec(const Rec64* p) {
	Rec64 r;
	const double2* s = reinterpret_cast<const double2*>(p);
	double2* d = reinterpret_cast<double2*>(&r);
#pragma unroll
	for (int i = 0; i < 8; i++) d[i] = __ldg(s + i);
	return r;
}
__device__ __forceinline__ Rec32 load_rec(const Rec32* p) {
	Rec32 r;
	const float4* s = reinterpret_cast<const float4*>(p);
	float4* d = reinterpret_cast<float4*>(&r);
#pragma unroll
	for (int i = 0; i < 5; i++) d[i] = __ldg(s + i);
	return r;
}
// the rest of a record whose first 16 bytes (x, y) are already loaded
__device__ __forceinline__ Rec32 load_rec_tail(const Rec32* p, float4 head) {
	Rec32 r;
	const float4* s = reinterpret_cast<const float4*>(p);
	float4* d = reinterpret_cast<float4*>(&r);
	d[0] = head;
#pragma unroll
	for (int i = 1; i < 5; i++) d[i] = __ldg(s + i);
	return r;
}

// ------------------------------------------------------- per-body failures
// With per-body masking (failed != nullptr) an error found on a row fails the row's
// body alone; without it, it fails the step (the status word).
__device__ __forceinline__ void fail_body(uint32_t* failed, DevStatus* st, uint32_t bit, uint32_t row, uint32_t body) {
	if (failed) atomicOr(&failed[body], bit);
	else raise(st, bit, row);
}
__device__ __forceinline__ bool is_failed(const uint32_t* failed, uint32_t body) {
	return failed && *(volatile const uint32_t*)&failed[body];
}

// --------------------------------------------------------------- grid build
__global__ void k_bbox_init(uint32_t nb, unsigned long long* bb) {
	uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= nb) return;
	bb[6 * b + 0] = ord_encode(1.7976931348623157e308);   // min x
	bb[6 * b + 1] = ord_encode(1.7976931348623157e308);   // min y
	bb[6 * b + 2] = ord_encode(-1.7976931348623157e308);  // max x
	bb[6 * b + 3] = ord_encode(-1.7976931348623157e308);  // max y
	bb[6 * b + 4] = ord_encode(-1.7976931348623157e308);  // h_max
	bb[6 * b + 5] = ord_encode(0.);                       // max |v|^2 (mixed form)
}

// Bounding box and h_max per body (grid.h:83-104).  Rows of a body are contiguous,
// so a warp whose rows share one body reduces in registers and issues one atomic
// per quantity.  The mixed form also takes the largest speed, which sizes cells that
// stay valid for all four stages of a step.
__global__ void k_bbox(uint32_t n, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ h, const double* __restrict__ vx, const double* __restrict__ vy,
                       const uint32_t* __restrict__ body_of, int mixed, unsigned long long* bb,
                       const uint32_t* failed) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	bool valid = i < n;
	uint32_t b = valid ? body_of[i] : 0xffffffffu;
	if (valid && is_failed(failed, b)) {  // a failed body's rows are left out
		valid = false;
		b = 0xffffffffu;
	}
	unsigned long long mnx = ~0ull, mny = ~0ull, mxx = 0ull, mxy = 0ull, mh = 0ull, mv = 0ull;
	if (valid) {
		mnx = mxx = ord_encode(x[i]);
		mny = mxy = ord_encode(y[i]);
		mh = ord_encode(h[i]);
		// the square of the speed (the square root once per body: a correctly rounded root
		// is monotonic, so the root of the largest square is the largest root)
		mv = mixed ? ord_encode(vx[i] * vx[i] + vy[i] * vy[i]) : ord_encode(0.);
	}
	uint32_t lane = threadIdx.x & 31;
	uint32_t b0 = __shfl_sync(0xffffffffu, b, 0);
	bool uniform = __all_sync(0xffffffffu, b == b0) && b0 != 0xffffffffu;
	if (uniform) {
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
			mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
			mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
			mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
			mh = max(mh, __shfl_xor_sync(0xffffffffu, mh, o));
			mv = max(mv, __shfl_xor_sync(0xffffffffu, mv, o));
		}
		if (lane == 0) {
			atomicMin(&bb[6 * b0 + 0], mnx);
			atomicMin(&bb[6 * b0 + 1], mny);
			atomicMax(&bb[6 * b0 + 2], mxx);
			atomicMax(&bb[6 * b0 + 3], mxy);
			atomicMax(&bb[6 * b0 + 4], mh);
			atomicMax(&bb[6 * b0 + 5], mv);
		}
	} else if (valid) {
		atomicMin(&bb[6 * b + 0], mnx);
		atomicMin(&bb[6 * b + 1], mny);
		atomicMax(&bb[6 * b + 2], mxx);
		atomicMax(&bb[6 * b + 3], mxy);
		atomicMax(&bb[6 * b + 4], mh);
		atomicMax(&bb[6 * b + 5], mv);
	}
}

// Cell geometry per body (grid.h:105-115) and the exclusive scan of cell counts.
// One block; bodies are processed serially in chunks for the scan.
__global__ void k_geom(uint32_t nb, const unsigned long long* bb, const BodyParams* P, int mixed, Geom* G,
                       uint32_t* total_cells, uint32_t cell_cap, DevStatus* st, uint32_t* failed) {
	__shared__ uint32_t s_cnt[1024];
	__shared__ uint32_t s_base;
	if (threadIdx.x == 0) s_base = 0;
	__syncthreads();
	for (uint32_t c0 = 0; c0 < nb; c0 += blockDim.x) {
		uint32_t b = c0 + threadIdx.x;
		uint32_t cnt = 0;
		Geom g{};
		if (b < nb && is_failed(failed, b)) {  // a failed body gets no cells
			g.nx = g.ny = 1;
			g.dx = 1.;
			g.span = 1;
		} else if (b < nb) {
			double bminx = ord_decode(bb[6 * b + 0]), bminy = ord_decode(bb[6 * b + 1]);
			double bmaxx = ord_decode(bb[6 * b + 2]), bmaxy = ord_decode(bb[6 * b + 3]);
			double hmax = ord_decode(bb[6 * b + 4]);
			bminx -= 1e-6; bminy -= 1e-6;
			bmaxx += 1e-6; bmaxy += 1e-6;
			double dx = hmax * 2.;
			double slack = 0.;
			uint32_t span = 1;
			double lx = bmaxx - bminx, ly = bmaxy - bminy;
			if (mixed) {
				// a particle moves at most ~ |v| dt per step; allow twice the fastest speed
				slack = 2. * sqrt(ord_decode(bb[6 * b + 5])) * P[b].dt;
				dx = 2. * hmax + 2. * slack;
				// half-size cells with a 5x5 stencil cover the same reach with ~40 % fewer
				// candidates than 3x3 cells of the full reach; used while the body's cells
				// stay below twice its particles
				double hx = 0.5 * dx;
				if (ceil(lx / hx) * ceil(ly / hx) <= 2.0 * P[b].n) {
					dx = hx;
					span = 2;
				}
			}
			double fnx = ceil(lx / dx), fny = ceil(ly / dx);
			uint32_t nx = (uint32_t)fnx, ny = (uint32_t)fny;
			uint32_t num_cell = nx * ny;
			bool bad = false;
			if (!(num_cell < P[b].n) && !mixed) {
				fail_body(failed, st, ERR_GRID, P[b].off, b);
				bad = true;
			}
			if (!(fnx * fny < 4.0e9) || nx == 0 || ny == 0) {
				fail_body(failed, st, ERR_GRID, P[b].off, b);
				nx = ny = 1;
				num_cell = 1;
				bad = true;
			}
			if (bad && failed) num_cell = 0;  // masked from this stage on
			g.bbmin_x = bminx; g.bbmin_y = bminy; g.dx = dx; g.slack = slack;
			g.nx = nx; g.ny = ny; g.num_cell = num_cell; g.span = span;
			cnt = num_cell;
		}
		s_cnt[threadIdx.x] = cnt;
		__syncthreads();
		if (threadIdx.x == 0) {
			uint32_t run = s_base;
			uint32_t lim = min((uint32_t)blockDim.x, nb - c0);
			for (uint32_t t = 0; t < lim; t++) {
				uint32_t c = s_cnt[t];
				s_cnt[t] = run;
				run += c;
			}
			s_base = run;
		}
		__syncthreads();
		if (b < nb) {
			g.cell_off = s_cnt[threadIdx.x];
			G[b] = g;
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		uint32_t tot = s_base;
		if (tot > cell_cap) {
			raise(st, ERR_GRID, 0);
			tot = 0;  // downstream kernels see an empty grid
		}
		*total_cells = tot;
	}
}

// Global cell key of each row (grid.h:35-41): cell_off + ix*ny + iy.
__global__ void k_hash(uint32_t n, const double* __restrict__ x, const double* __restrict__ y,
                       const uint32_t* __restrict__ body_of, const Geom* __restrict__ G,
                       const uint32_t* __restrict__ total_cells, uint32_t* keys, uint32_t* vals, DevStatus* st,
                       uint32_t* failed) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t b = body_of[i], tot = *total_cells;
	vals[i] = i;
	if (is_failed(failed, b) && tot != 0) {  // past every cell: no stencil reaches it
		keys[i] = tot;
		return;
	}
	Geom g = G[b];
	uint32_t ix = (uint32_t)((x[i] - g.bbmin_x) / g.dx);
	uint32_t iy = (uint32_t)((y[i] - g.bbmin_y) / g.dx);
	if (ix >= g.nx || iy >= g.ny || tot == 0) {
		if (tot != 0 && failed) {
			atomicOr(&failed[b], ERR_GRID);
			keys[i] = tot;
			return;
		}
		raise(st, ERR_GRID, i);
		ix = min(ix, g.nx - 1);
		iy = min(iy, g.ny - 1);
	}
	uint32_t key = g.cell_off + ix * g.ny + iy;
	keys[i] = (tot == 0) ? 0u : key;
}

// Cell start table over all bodies' cells (grid.h:48-81): cell_start[c] is the
// first sorted position with key >= c, so empty cells get the next start.
__global__ void k_cells(uint32_t n, const uint32_t* __restrict__ keys, const uint32_t* __restrict__ total_cells,
                        uint32_t* cell_start) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t tot = *total_cells;
	if (k > n) return;
	if (k == n) {
		uint32_t last = (n == 0) ? 0u : keys[n - 1] + 1;
		for (uint32_t c = last; c <= tot; c++) cell_start[c] = n;
		return;
	}
	uint32_t key = min(keys[k], tot);
	uint32_t prev = (k == 0) ? 0u : min(keys[k - 1], tot) + 1;
	if (k == 0 || keys[k] != keys[k - 1])
		for (uint32_t c = prev; c <= key; c++) cell_start[c] = k;
}

// ---------------------------------------------------------------- gather
template <bool MIXED>
struct StageView;

// Reads the stage state of row i: stage 0 reads the base state (k1 is a copy of
// the particles, rk4.h:76-78), later stages the RK stage arrays.
template <>
struct StageView<false> {
	const double *x, *y, *vx, *vy, *rho, *Sxx, *Sxy, *Syy;
	__device__ void load(uint32_t i, double& X, double& Y, double& VX, double& VY, double& R, double& A, double& B,
	                     double& C) const {
		X = x[i]; Y = y[i]; VX = vx[i]; VY = vy[i]; R = rho[i]; A = Sxx[i]; B = Sxy[i]; C = Syy[i];
	}
};
template <>
struct StageView<true> {
	const double *x, *y, *vx, *vy;
	const float *rho, *Sxx, *Sxy, *Syy;
	__device__ void load(uint32_t i, double& X, double& Y, double& VX, double& VY, float& R, float& A, float& B,
	                     float& C) const {
		X = x[i]; Y = y[i]; VX = vx[i]; VY = vy[i]; R = rho[i]; A = Sxx[i]; B = Sxy[i]; C = Syy[i];
	}
};

template <bool MIXED>
__device__ StageView<MIXED> stage_view(const ULArgs& a);
template <>
__device__ StageView<false> stage_view<false>(const ULArgs& a) {
	const mfk_host::StateSoA& s = a.stage == 0 ? a.base : a.st;
	return StageView<false>{s.x, s.y, s.vx, s.vy, s.rho, s.Sxx, s.Sxy, s.Syy};
}
template <>
__device__ StageView<true> stage_view<true>(const ULArgs& a) {
	const mfk_host::StateSoA& s = a.stage == 0 ? a.base : a.st;
	return StageView<true>{s.x, s.y, s.vx, s.vy, s.rho_f, s.Sxx_f, s.Sxy_f, s.Syy_f};
}

// Per-particle actions of one stage: EOS, artificial stress, integration weight.
template <class T>
__device__ __forceinline__ void per_particle(uint32_t flags, const BodyParams& pr, T m, T rho, T qw0, T Sxx, T Sxy,
                                             T Syy, T& sxx_o, T& syy_o, T& Rxx, T& Rxy, T& Ryy, T& c, T& qw,
                                             T& rho21) {
	T p = T(0);
	if (flags & A_EOS) p = T(pr.c0sq) * (rho - T(pr.rho0));  // c0*c0*(rho - rho0)
	T sxx = Sxx - p, syy = Syy - p, sxy = Sxy;
	Rxx = Rxy = Ryy = T(0);
	if (flags & A_ART_STRESS) {
		T eps = T(pr.mghn_eps);
		T theta = T(0.5) * atan2(T(2.) * sxy, sxx - syy + T(0.));
		T cs = cos(theta), sn = sin(theta);
		T cs2 = cs * cs, sn2 = sn * sn;
		T rot_sxx = cs2 * sxx + T(2.0) * cs * sn * sxy + sn2 * syy;
		T rot_syy = sn2 * sxx - T(2.0) * cs * sn * sxy + cs2 * syy;
		T rot_rxx = T(0), rot_ryy = T(0);
		if (rot_sxx > T(0)) rot_rxx = -eps * rot_sxx / (rho * rho);
		if (rot_syy > T(0)) rot_ryy = -eps * rot_syy / (rho * rho);
		Rxx = cs2 * rot_rxx + sn2 * rot_ryy;
		Rxy = cs * sn * (rot_rxx - rot_ryy);
		Ryy = sn2 * rot_rxx + cs2 * rot_ryy;
	}
	sxx_o = sxx;
	syy_o = syy;
	c = sqrt(T(pr.K) / rho);
	qw = (flags & A_RIEMANN) ? m / rho : qw0;
	rho21 = T(1.) / (rho * rho);
}

// The same in FP32 for the mixed gather, from the parameters' FP32 copies, the EOS from
// the stored rho - rho0 (no cancellation of rho - rho0 in FP32)
__device__ __forceinline__ void per_particle32(uint32_t flags, const BodyParams& pr, float m, float rho, float drho,
                                               float qw0, float Sxx, float Sxy, float Syy, float& sxx_o, float& syy_o,
                                               float& Rxx, float& Rxy, float& Ryy, float& c, float& qw,
                                               float& rho21) {
	float p = 0.f;
	if (flags & A_EOS) p = pr.fc0sq * drho;
	float sxx = Sxx - p, syy = Syy - p, sxy = Sxy;
	Rxx = Rxy = Ryy = 0.f;
	if (flags & A_ART_STRESS) {
		float eps = pr.fmghn_eps;
		float theta = 0.5f * atan2f(2.f * sxy, sxx - syy + 0.f);
		float cs = cosf(theta), sn = sinf(theta);
		float cs2 = cs * cs, sn2 = sn * sn;
		float rot_sxx = cs2 * sxx + 2.f * cs * sn * sxy + sn2 * syy;
		float rot_syy = sn2 * sxx - 2.f * cs * sn * sxy + cs2 * syy;
		float rot_rxx = 0.f, rot_ryy = 0.f;
		if (rot_sxx > 0.f) rot_rxx = -eps * rot_sxx / (rho * rho);
		if (rot_syy > 0.f) rot_ryy = -eps * rot_syy / (rho * rho);
		Rxx = cs2 * rot_rxx + sn2 * rot_ryy;
		Rxy = cs * sn * (rot_rxx - rot_ryy);
		Ryy = sn2 * rot_rxx + cs2 * rot_ryy;
	}
	sxx_o = sxx;
	syy_o = syy;
	c = sqrtf(pr.fK / rho);
	qw = (flags & A_RIEMANN) ? m / rho : qw0;
	rho21 = 1.f / (rho * rho);
}

__global__ void k_gather64(ULArgs a, const BodyParams* __restrict__ P) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.n_total) return;
	uint32_t i = a.perm[k];
	StageView<false> v = stage_view<false>(a);
	double x, y, vx, vy, rho, Sxx, Sxy, Syy;
	v.load(i, x, y, vx, vy, rho, Sxx, Sxy, Syy);
	uint32_t b = a.body_of[i];
	Rec64 r;
	r.x = x; r.y = y; r.vx = vx; r.vy = vy;
	r.m = a.m[i]; r.h = a.h[i]; r.rho = rho;
	per_particle<double>(a.flags, P[b], r.m, rho, a.qw0[i], Sxx, Sxy, Syy, r.sxx, r.syy, r.Rxx, r.Rxy, r.Ryy, r.c, r.qw,
	                     r.rho21);
	r.sxy = Sxy;
	if (a.flags & (A_GOD_CONT | A_GOD_MOM)) {
		r.Rxx = (a.flags & A_EOS) ? P[b].c0sq * (rho - P[b].rho0) : 0.;
		r.Rxy = Syy;
	}
	Rec64* out = reinterpret_cast<Rec64*>(a.rec) + k;
	const double2* s = reinterpret_cast<const double2*>(&r);
	double2* d = reinterpret_cast<double2*>(out);
#pragma unroll
	for (int q = 0; q < 8; q++) d[q] = s[q];
	a.rec_body[k] = b;
}

// The record of particle i (body parameters pr) from its stage state, into out.
__device__ __forceinline__ void put_rec32(const ULArgs& a, const BodyParams& pr, uint32_t i, Rec32* out, double x,
                                          double y, double vx, double vy, float rho_dev, float Sxx, float Sxy,
                                          float Syy) {
	const float rho = rho_dev + pr.frho0;  // the mixed state holds rho - rho0
	Rec32 r;
	r.x = ff_split_bits(x); r.y = ff_split_bits(y); r.vx = ff_split_bits(vx); r.vy = ff_split_bits(vy);
	r.m = (float)a.m[i]; r.h = (float)a.h[i]; r.rho = rho;
	per_particle32(a.flags, pr, r.m, rho, rho_dev, (float)a.qw0[i], Sxx, Sxy, Syy, r.sxx, r.syy, r.Rxx, r.Rxy, r.Ryy,
	               r.c, r.qw, r.rho21);
	r.sxy = Sxy;
	if (a.flags & (A_GOD_CONT | A_GOD_MOM)) {  // p from the stored deviation, the stress Syy itself
		r.Rxx = (a.flags & A_EOS) ? pr.fc0sq * rho_dev : 0.f;
		r.Rxy = Syy;
	}
	const float4* s = reinterpret_cast<const float4*>(&r);
	float4* d = reinterpret_cast<float4*>(out);
#pragma unroll
	for (int q = 0; q < 5; q++) d[q] = s[q];
}

__global__ void k_gather32(ULArgs a, const BodyParams* __restrict__ P) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.n_total) return;
	uint32_t i = a.perm[k];
	StageView<true> v = stage_view<true>(a);
	double x, y, vx, vy;
	float rho, Sxx, Sxy, Syy;
	v.load(i, x, y, vx, vy, rho, Sxx, Sxy, Syy);
	uint32_t b = a.body_of[i];
	put_rec32(a, P[b], i, reinterpret_cast<Rec32*>(a.rec) + k, x, y, vx, vy, rho, Sxx, Sxy, Syy);
	a.rec_body[k] = b;
}

// --------------------------------------------------------------- RK update
// rk4.h:52-69 (stage state = particles + c*dt*derivative) and :94-103 (final
// combine with weights 1,2,2,1 / 6).  d[] = x_t, y_t, vx_t, vy_t, rho_t, Sxx_t, Sxy_t, Syy_t.
template <class T>
__device__ __forceinline__ void rk_update_f64(const ULArgs& a, uint32_t i, double dt, const double d[8]) {
	double* bp[8] = {a.base.x, a.base.y, a.base.vx, a.base.vy, a.base.rho, a.base.Sxx, a.base.Sxy, a.base.Syy};
	double* ap[8] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy, a.acc.rho, a.acc.Sxx, a.acc.Sxy, a.acc.Syy};
	double* sp[8] = {a.st.x, a.st.y, a.st.vx, a.st.vy, a.st.rho, a.st.Sxx, a.st.Sxy, a.st.Syy};
	uint32_t s = a.stage;
	if (s < 3) {
		double dts = (s == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q = 0; q < 8; q++) {
			double accv = (s == 0) ? d[q] : ap[q][i] + 2 * d[q];
			ap[q][i] = accv;
			sp[q][i] = bp[q][i] + d[q] * dts;
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 8; q++) bp[q][i] = bp[q][i] + w6 * (ap[q][i] + d[q]);
	}
}

// Mixed form: x, y, vx, vy accumulate in FP64, rho and the stresses in FP32.
__device__ __forceinline__ void rk_update_mixed(const ULArgs& a, uint32_t i, double dt, const float d[8]) {
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* sp[4] = {a.st.x, a.st.y, a.st.vx, a.st.vy};
	float* bq[4] = {a.base.rho_f, a.base.Sxx_f, a.base.Sxy_f, a.base.Syy_f};
	float* aq[4] = {a.acc.rho_f, a.acc.Sxx_f, a.acc.Sxy_f, a.acc.Syy_f};
	float* sq[4] = {a.st.rho_f, a.st.Sxx_f, a.st.Sxy_f, a.st.Syy_f};
	uint32_t s = a.stage;
	if (s < 3) {
		double dts = (s == 2 ? 1.0 : 0.5) * dt;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			double dq = (double)d[q];
			ap[q][i] = (s == 0) ? dq : ap[q][i] + 2 * dq;
			sp[q][i] = bp[q][i] + dq * dts;
			float dr = d[4 + q];
			aq[q][i] = (s == 0) ? dr : aq[q][i] + 2.f * dr;
			sq[q][i] = bq[q][i] + dr * (float)dts;
		}
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			bp[q][i] = bp[q][i] + w6 * (ap[q][i] + (double)d[q]);
			bq[q][i] = bq[q][i] + (float)w6 * (aq[q][i] + d[4 + q]);
		}
	}
}

__device__ __forceinline__ void stencil(const Geom& g, uint32_t key, int& lo_i, int& hi_i, int& lo_j, int& hi_j) {
	uint32_t b = key - g.cell_off;
	uint32_t gi = b / g.ny;
	uint32_t gj = b - gi * g.ny;
	const int sp = (int)g.span;
	lo_i = (int)gi - sp < 0 ? 0 : (int)gi - sp;
	lo_j = (int)gj - sp < 0 ? 0 : (int)gj - sp;
	hi_i = (int)gi + sp + 1 > (int)g.nx ? (int)g.nx : (int)gi + sp + 1;
	hi_j = (int)gj + sp + 1 > (int)g.ny ? (int)g.ny : (int)gj + sp + 1;
}

// ----------------------------------------------------------- pair kernel FP64
__device__ __forceinline__ void pair64_row(const ULArgs& a, const BodyParams* __restrict__ P,
                                           const Geom* __restrict__ G, DevStatus* st, uint32_t k) {
	uint32_t b = a.rec_body[k];
	if (is_failed(a.failed, b)) return;  // a failed body stays as it was
	const Rec64* rec = reinterpret_cast<const Rec64*>(a.rec);
	const Rec64 ri = load_rec(rec + k);
	const BodyParams& pr = P[b];
	Geom g = G[b];
	uint32_t i = a.perm[k];
	uint32_t flags = a.flags;
	int lo_i, hi_i, lo_j, hi_j;
	stencil(g, a.keys_sorted[k], lo_i, hi_i, lo_j, hi_j);
	const uint32_t tot = *a.total_cells;

	double hi = ri.h;
	double radius2 = __dmul_rn(__dmul_rn(__dmul_rn(hi, hi), 2.), 2.);
	double lim = __dadd_rn(radius2, a.nbh_eps);
	double reach2 = 4.0000001 * hi * hi;  // pairs beyond q = 2 contribute exactly zero
	double rhoi21 = ri.rho21;
	double wdeltap = pr.wdeltap, corr_exp = pr.corr_exp;
	double alpha = pr.alpha, beta = pr.beta, eta = pr.eta, xeps = pr.xsph_eps;

	double Sxx_x = 0., Sxy_y = 0., Sxy_x = 0., Syy_y = 0.;
	double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0.;
	double av_x = 0., av_y = 0., xs_x = 0., xs_y = 0.;
	double god_rho = 0., god_vx = 0., god_vy = 0.;
	const double two_rhoi = 2. / ri.rho;  // godunov.h:127-133's 2./rhoi, the same per pair
	uint32_t cnt = 0;
	for (int ni = lo_i; ni < hi_i; ni++) {
		uint32_t c0 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)lo_j, tot);
		uint32_t c1 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)hi_j, tot);
		uint32_t j0 = a.cell_start[c0], j1 = a.cell_start[c1];
		for (uint32_t kj = j0; kj < j1; kj++) {
			const Rec64 rj = load_rec(rec + kj);
			double xij = __dsub_rn(ri.x, rj.x);
			double yij = __dsub_rn(ri.y, rj.y);
			double r2 = __dadd_rn(__dmul_rn(xij, xij), __dmul_rn(yij, yij));
			cnt += (r2 <= lim) ? 1u : 0u;
			if (r2 > reach2) continue;
			KR64 w = cubic_spline(xij, yij, hi);
			if (flags & A_STRESS_MGHN) {
				double Rxx = 0., Rxy = 0., Ryy = 0.;
				if (wdeltap > 0) {
					double fab = w.w / wdeltap;
					if (corr_exp == 4.) {
						double f2 = fab * fab;
						fab = f2 * f2;
					} else {
						fab = pow(fab, corr_exp);
					}
					Rxx = fab * (ri.Rxx + rj.Rxx);
					Rxy = fab * (ri.Rxy + rj.Rxy);
					Ryy = fab * (ri.Ryy + rj.Ryy);
				}
				Sxx_x += rj.m * (ri.sxx * rhoi21 + rj.sxx * rj.rho21 + Rxx) * w.w_x;
				Sxy_y += rj.m * (ri.sxy * rhoi21 + rj.sxy * rj.rho21 + Rxy) * w.w_y;
				Sxy_x += rj.m * (ri.sxy * rhoi21 + rj.sxy * rj.rho21 + Rxy) * w.w_x;
				Syy_y += rj.m * (ri.syy * rhoi21 + rj.syy * rj.rho21 + Ryy) * w.w_y;
			}
			if (flags & A_DERIVE_VEL) {
				vx_x += (rj.vx - ri.vx) * w.w_x * rj.qw;
				vx_y += (rj.vx - ri.vx) * w.w_y * rj.qw;
				vy_x += (rj.vy - ri.vy) * w.w_x * rj.qw;
				vy_y += (rj.vy - ri.vy) * w.w_y * rj.qw;
			}
			double vijx = ri.vx - rj.vx, vijy = ri.vy - rj.vy;
			if (flags & A_ART_VISC) {
				double vijposij = vijx * xij + vijy * yij;
				if (vijposij < 0.) {
					double cij = 0.5 * (ri.c + rj.c);
					double hij = 0.5 * (hi + rj.h);
					double rhoij = 0.5 * (ri.rho + rj.rho);
					double r2ij = xij * xij + yij * yij;
					double muij = (hij * vijposij) / (r2ij + eta * eta * hij * hij);
					double piij = (-alpha * cij * muij + beta * muij * muij) / rhoij;
					av_x += -rj.m * piij * w.w_x;
					av_y += -rj.m * piij * w.w_y;
				}
			}
			if (flags & A_XSPH) {
				double rhoij = 0.5 * (ri.rho + rj.rho);
				double fac = -xeps * w.w * ri.m / rhoij;
				xs_x += fac * vijx;
				xs_y += fac * vijy;
			}
			if ((flags & (A_GOD_CONT | A_GOD_MOM)) && kj != k) {
				// |x_j - x_i| from the predicate's own sum (the same value as the
				// reference's sqrt(dx*dx + dy*dy) and sqrt(dot(R, R)))
				const double mag_r = sqrt(r2);
				// the acoustic Riemann denominator, the same expression in both actions
				const double frac = 1. / (ri.rho * ri.c + rj.rho * rj.c);
#if !MF_STRICT_FORM
				const double inv_r = 1. / mag_r;
#endif
				if (flags & A_GOD_CONT) {  // godunov_continuity, godunov.h:144-187
#if MF_STRICT_FORM
					double nx = xij / mag_r, ny = yij / mag_r;
#else
					double nx = xij * inv_r, ny = yij * inv_r;
#endif
					double vir = ri.vx * nx + ri.vy * ny;
					double vjr = rj.vx * nx + rj.vy * ny;
					// riemann_solver_acoustic (godunov.h:41-54); Rxx = p
					double ustar = frac * (vir * ri.rho * ri.c + vjr * rj.rho * rj.c - ri.Rxx + rj.Rxx);
					god_rho += 2 * ri.rho * (vir - ustar) * (w.w_x * nx + w.w_y * ny) * rj.qw;
				}
				if (flags & A_GOD_MOM) {  // godunov_get_trafo + godunov_momentum, godunov.h:56-142
					double rx = rj.x - ri.x, ry = rj.y - ri.y;
#if MF_STRICT_FORM
					double inv = 1. / mag_r;  // glm::normalize: v * (1 / sqrt(dot(v, v)))
#else
					double inv = inv_r;
#endif
					double Rx = rx * inv, Ry = ry * inv, Sx = ry * inv, Sy = -rx * inv;
					// the frame matrix is single precision (a glm::mat2x2 of the unit vectors)
					double lRx = (double)__double2float_rn(Rx), lRy = (double)__double2float_rn(Ry);
					double lSx = (double)__double2float_rn(Sx), lSy = (double)__double2float_rn(Sy);
					// stress times R: (Sxx - p, Sxy; Sxy, Syy), Rxy = Syy
					double siR0 = ri.sxx * Rx + ri.sxy * Ry, siR1 = ri.sxy * Rx + ri.Rxy * Ry;
					double sjR0 = rj.sxx * Rx + rj.sxy * Ry, sjR1 = rj.sxy * Rx + rj.Rxy * Ry;
					double si0 = lRx * siR0 + lSx * siR1;
					double sj0 = lRx * sjR0 + lSx * sjR1, sj1 = lRy * sjR0 + lSy * sjR1;
					double vi0 = lRx * ri.vx + lSx * ri.vy, vi1 = lRy * ri.vx + lSy * ri.vy;
					double vj0 = lRx * rj.vx + lSx * rj.vy, vj1 = lRy * rj.vx + lSy * rj.vy;
					// the second component takes sigma_j twice (godunov.h:116), as the reference does
					double S0 = frac * (sj0 * ri.rho * ri.c + si0 * rj.rho * rj.c + ri.rho * ri.c * rj.rho * rj.c * (vj0 - vi0));
					double S1 = frac * (sj1 * ri.rho * ri.c + sj1 * rj.rho * rj.c + ri.rho * ri.c * rj.rho * rj.c * (vj1 - vi1));
					double SR0 = lRx * S0 + lRy * S1, SR1 = lSx * S0 + lSy * S1;
					if (fabs(rx) > 0.) god_vx += two_rhoi * w.w_x * mag_r / rx * SR0 * rj.qw;
					if (fabs(ry) > 0.) god_vy += two_rhoi * w.w_y * mag_r / ry * SR1 * rj.qw;
				}
			}
		}
	}
	if (a.max_nbh && cnt >= a.max_nbh) fail_body(a.failed, st, ERR_NBH_OVERFLOW, i, b);
	if (cnt == 0) fail_body(a.failed, st, ERR_NO_NEIGHBOR, i, b);

	// per-particle actions, in the reference's list order
	double d[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
	double rhoi = ri.rho;
	if (flags & A_STRESS_MGHN) { Sxx_x *= rhoi; Sxy_y *= rhoi; Sxy_x *= rhoi; Syy_y *= rhoi; }
	if (flags & A_ART_VISC) { d[2] = av_x; d[3] = av_y; }
	if (flags & A_XSPH) { d[0] = xs_x; d[1] = xs_y; }
	if (flags & A_JAUMANN) {
		// the Jaumann rate uses the stage stress itself (not S - p)
		const mfk_host::StateSoA& sv = a.stage == 0 ? a.base : a.st;
		jaumann<double>(vx_x, vx_y, vy_x, vy_y, sv.Sxx[i], sv.Sxy[i], sv.Syy[i], pr.G, d[5], d[6], d[7]);
	}
	if (flags & A_CONTINUITY) d[4] = -(rhoi * (vx_x + vy_y));
	if (flags & A_GOD_CONT) d[4] = god_rho;
	if (flags & A_GOD_MOM) {
		d[2] += god_vx + a.fcx[i] / ri.m;
		d[3] += god_vy + a.fcy[i] / ri.m;
	}
	if (flags & A_MOMENTUM_UL) {
		d[2] += 1. / rhoi * (Sxx_x + Sxy_y) + a.fcx[i] / ri.m;
		d[3] += 1. / rhoi * (Sxy_x + Syy_y) + a.fcy[i] / ri.m;
	}
	if (flags & A_ADVECTION) { d[0] += ri.vx; d[1] += ri.vy; }
	rk_update_f64<double>(a, i, pr.dt, d);
	if (a.stage == 3 && !(isfinite(a.base.x[i]) && isfinite(a.base.y[i]) && isfinite(a.base.vx[i]) &&
	                      isfinite(a.base.vy[i]) && isfinite(a.base.rho[i])))
		fail_body(a.failed, st, ERR_NONFINITE, i, b);
}

// ---------------------------------------------------------- pair kernel mixed
// L threads per row (L = 1: one thread walks the row's whole stencil): lane takes every
// L-th candidate of each stencil row, the partial sums are added across the L lanes,
// and lane 0 finishes the row.  L > 1 puts more rows' work in flight when the rows are
// few (the launch would otherwise cover a handful of SMs); it changes the order of the
// pair sums, not their terms.
template <bool GOD, int L = 1>
__device__ __forceinline__ void pair32_row(const ULArgs& a, const BodyParams* __restrict__ P,
                                           const Geom* __restrict__ G, DevStatus* st, uint32_t k,
                                           uint32_t lane = 0) {
	uint32_t b = a.rec_body[k];
	if (is_failed(a.failed, b)) return;  // a failed body stays as it was (all L lanes of the row)
	const Rec32* rec = reinterpret_cast<const Rec32*>(a.rec);
	const Rec32 ri = load_rec(rec + k);
	const BodyParams& pr = P[b];
	Geom g = G[b];
	uint32_t i = a.perm[k];
	uint32_t flags = a.flags;
	int lo_i, hi_i, lo_j, hi_j;
	stencil(g, a.keys_sorted[k], lo_i, hi_i, lo_j, hi_j);
	const uint32_t tot = *a.total_cells;

	float hi = ri.h;
	float h1 = 1.f / hi;
	float fac = (float)(10 * (K_1_PI) / 7.0) * h1 * h1;
	float reach2 = 4.0001f * hi * hi;
	float rhoi21 = ri.rho21;
	// the parameters' FP32 copies: a conversion (let alone a division) in FP64 would run
	// on the narrow FP64 pipe for every row
	float wdp1 = pr.fwdp1;
	bool exp4 = pr.fcorr_exp == 4.f;
	float corr_exp = pr.fcorr_exp;
	float alpha = pr.falpha, beta = pr.fbeta, eta2 = pr.feta2, xeps = pr.fxsph_eps;

	float Sxx_x = 0.f, Sxy_y = 0.f, Sxy_x = 0.f, Syy_y = 0.f;
	float vx_x = 0.f, vx_y = 0.f, vy_x = 0.f, vy_y = 0.f;
	float av_x = 0.f, av_y = 0.f, xs_x = 0.f, xs_y = 0.f;
	float god_rho = 0.f, god_vx = 0.f, god_vy = 0.f;
	const float two_rhoi = 2.f / ri.rho;
	// the pair terms of candidate kj within reach (xij, yij: x_i - x_j; r2 = |x_i - x_j|^2)
	auto pair = [&](uint32_t kj, float4 head, float xij, float yij, float r2) {
		const Rec32 rj = load_rec_tail(rec + kj, head);
		KR32 w = cubic_spline_f(xij, yij, h1, fac);
		if (flags & A_STRESS_MGHN) {
			float Rxx = 0.f, Rxy = 0.f, Ryy = 0.f;
			if (wdp1 > 0.f) {
				float fab = w.w * wdp1;
				if (exp4) {
					float f2 = fab * fab;
					fab = f2 * f2;
				} else {
					fab = powf(fab, corr_exp);
				}
				Rxx = fab * (ri.Rxx + rj.Rxx);
				Rxy = fab * (ri.Rxy + rj.Rxy);
				Ryy = fab * (ri.Ryy + rj.Ryy);
			}
			float tsx = rj.m * (ri.sxy * rhoi21 + rj.sxy * rj.rho21 + Rxy);
			Sxx_x += rj.m * (ri.sxx * rhoi21 + rj.sxx * rj.rho21 + Rxx) * w.w_x;
			Sxy_y += tsx * w.w_y;
			Sxy_x += tsx * w.w_x;
			Syy_y += rj.m * (ri.syy * rhoi21 + rj.syy * rj.rho21 + Ryy) * w.w_y;
		}
		float dvx = ff_diff(rj.vx, ri.vx), dvy = ff_diff(rj.vy, ri.vy);
		if (flags & A_DERIVE_VEL) {
			float qx = w.w_x * rj.qw, qy = w.w_y * rj.qw;
			vx_x += dvx * qx;
			vx_y += dvx * qy;
			vy_x += dvy * qx;
			vy_y += dvy * qy;
		}
		if (flags & A_ART_VISC) {
			float vijposij = -(dvx * xij + dvy * yij);
			if (vijposij < 0.f) {
				float cij = 0.5f * (ri.c + rj.c);
				float hij = 0.5f * (hi + rj.h);
				float rhoij = 0.5f * (ri.rho + rj.rho);
				float muij = __fdividef(hij * vijposij, r2 + eta2 * hij * hij);
				float piij = __fdividef(-alpha * cij * muij + beta * muij * muij, rhoij);
				av_x += -rj.m * piij * w.w_x;
				av_y += -rj.m * piij * w.w_y;
			}
		}
		if (flags & A_XSPH) {
			float rhoij = 0.5f * (ri.rho + rj.rho);
			float f = __fdividef(-xeps * w.w * ri.m, rhoij);
			xs_x -= f * dvx;
			xs_y -= f * dvy;
		}
		if (GOD && kj != k) {
			// godunov_continuity / godunov_momentum (godunov.h:86-187) in FP32: velocity
			// differences from the float-float records, the Riemann state in the form
			// v_i - u* = (Z_j (v_i - v_j).n + p_i - p_j) / (Z_i + Z_j), Z = rho c;
			// Rxx holds p, Rxy the stress Syy itself
			const float mag_r = sqrtf(r2), inv = 1.f / mag_r;
			const float Zi = ri.rho * ri.c, Zj = rj.rho * rj.c;
			const float frac = 1.f / (Zi + Zj);
			if (flags & A_GOD_CONT) {
				float nx = xij * inv, ny = yij * inv;
				float dvn = -(dvx * nx + dvy * ny);  // (v_i - v_j).n
				float vi_us = frac * (Zj * dvn + (ri.Rxx - rj.Rxx));
				god_rho += 2.f * ri.rho * vi_us * (w.w_x * nx + w.w_y * ny) * rj.qw;
			}
			if (flags & A_GOD_MOM) {
				float rx = -xij, ry = -yij;
				float Rx = rx * inv, Ry = ry * inv, Sx = ry * inv, Sy = -rx * inv;  // the float frame
				float siR0 = ri.sxx * Rx + ri.sxy * Ry;
				float sjR0 = rj.sxx * Rx + rj.sxy * Ry, sjR1 = rj.sxy * Rx + rj.Rxy * Ry;
				float si0 = Rx * siR0 + Sx * (ri.sxy * Rx + ri.Rxy * Ry);
				float sj0 = Rx * sjR0 + Sx * sjR1, sj1 = Ry * sjR0 + Sy * sjR1;
				float dv0 = Rx * dvx + Sx * dvy, dv1 = Ry * dvx + Sy * dvy;  // frame (v_j - v_i)
				// the second component takes sigma_j twice (godunov.h:116), as the reference does
				float S0 = frac * (sj0 * Zi + si0 * Zj + Zi * Zj * dv0);
				float S1 = frac * (sj1 * Zi + sj1 * Zj + Zi * Zj * dv1);
				float SR0 = Rx * S0 + Ry * S1, SR1 = Sx * S0 + Sy * S1;
				if (fabsf(rx) > 0.f) god_vx += two_rhoi * __fdividef(w.w_x * mag_r, rx) * SR0 * rj.qw;
				if (fabsf(ry) > 0.f) god_vy += two_rhoi * __fdividef(w.w_y * mag_r, ry) * SR1 * rj.qw;
			}
		}
	};
	// candidate offsets and squared distance, one rounding each (the same values in both
	// walks below)
	auto offs = [&](float4 head, float& xij, float& yij) {
		xij = __fadd_rn(__fsub_rn(ri.x.hi, head.x), __fsub_rn(ri.x.lo, head.y));
		yij = __fadd_rn(__fsub_rn(ri.y.hi, head.z), __fsub_rn(ri.y.lo, head.w));
		return __fmaf_rn(yij, yij, __fmul_rn(xij, xij));
	};
	for (int ni = lo_i; ni < hi_i; ni++) {
		uint32_t c0 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)lo_j, tot);
		uint32_t c1 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)hi_j, tot);
		uint32_t j0 = a.cell_start[c0], j1 = a.cell_start[c1];
		if (L == 1 && j1 - j0 <= 32u) {
			// this stencil column's candidates tested first, into one mask, then the pair
			// terms of those within reach in ascending order: a warp runs as many pair
			// evaluations as its lane with the most neighbours in the column, instead of one
			// for every candidate that some lane accepts (the same pairs in the same order)
			uint32_t mask = 0u;
			for (uint32_t kj = j0; kj < j1; kj++) {
				float xij, yij;
				const float r2 = offs(__ldg(reinterpret_cast<const float4*>(rec + kj)), xij, yij);
				if (!(r2 > reach2)) mask |= 1u << (kj - j0);
			}
			while (mask) {
				const uint32_t kj = j0 + (uint32_t)(__ffs(mask) - 1);
				mask &= mask - 1u;
				const float4 head = __ldg(reinterpret_cast<const float4*>(rec + kj));
				float xij, yij;
				const float r2 = offs(head, xij, yij);
				pair(kj, head, xij, yij, r2);
			}
		} else {
			for (uint32_t kj = j0 + lane; kj < j1; kj += L) {
				// positions first: most candidates of the stencil lie beyond the reach
				const float4 head = __ldg(reinterpret_cast<const float4*>(rec + kj));
				float xij, yij;
				const float r2 = offs(head, xij, yij);
				if (r2 > reach2) continue;
				pair(kj, head, xij, yij, r2);
			}
		}
	}
	if (L > 1) {
		const unsigned gmask = ((1u << L) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(L - 1));
		float* acc[15] = {&Sxx_x, &Sxy_y, &Sxy_x, &Syy_y, &vx_x, &vx_y, &vy_x, &vy_y,
		                  &av_x, &av_y, &xs_x, &xs_y, &god_rho, &god_vx, &god_vy};
#pragma unroll
		for (int q = 0; q < 15; q++)
#pragma unroll
			for (int o = L / 2; o > 0; o >>= 1) *acc[q] += __shfl_xor_sync(gmask, *acc[q], o, L);
		if (lane != 0) return;
	}
	float d[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	float rhoi = ri.rho;
	if (flags & A_STRESS_MGHN) { Sxx_x *= rhoi; Sxy_y *= rhoi; Sxy_x *= rhoi; Syy_y *= rhoi; }
	if (flags & A_ART_VISC) { d[2] = av_x; d[3] = av_y; }
	if (flags & A_XSPH) { d[0] = xs_x; d[1] = xs_y; }
	float vxi = ri.vx.hi + ri.vx.lo, vyi = ri.vy.hi + ri.vy.lo;
	if (flags & A_JAUMANN) {
		const mfk_host::StateSoA& sv = a.stage == 0 ? a.base : a.st;
		jaumann<float>(vx_x, vx_y, vy_x, vy_y, sv.Sxx_f[i], sv.Sxy_f[i], sv.Syy_f[i], pr.fG, d[5], d[6], d[7]);
	}
	if (flags & A_CONTINUITY) d[4] = -(rhoi * (vx_x + vy_y));
	if (GOD && (flags & A_GOD_CONT)) d[4] = god_rho;
	if (GOD && (flags & A_GOD_MOM)) {
		d[2] += god_vx + (float)a.fcx[i] / ri.m;
		d[3] += god_vy + (float)a.fcy[i] / ri.m;
	}
	if (flags & A_MOMENTUM_UL) {
		d[2] += 1.f / rhoi * (Sxx_x + Sxy_y) + (float)a.fcx[i] / ri.m;
		d[3] += 1.f / rhoi * (Sxy_x + Syy_y) + (float)a.fcy[i] / ri.m;
	}
	if (a.stage > 0) {
		// the cells were sized at stage 0 for moves up to g.slack; check that held
		double mx = a.st.x[i] - a.base.x[i], my = a.st.y[i] - a.base.y[i];
		if (mx * mx + my * my > g.slack * g.slack) fail_body(a.failed, st, ERR_GRID, i, b);
	}
	// advection: the FP64 velocity enters the FP64 position update below
	double dd0 = (double)d[0], dd1 = (double)d[1];
	if (flags & A_ADVECTION) {
		const mfk_host::StateSoA& s = a.stage == 0 ? a.base : a.st;
		dd0 += s.vx[i];
		dd1 += s.vy[i];
	}
	(void)vxi; (void)vyi;
	// position/velocity in FP64, rho/S in FP32
	uint32_t s = a.stage;
	double dt = pr.dt;
	double dq[4] = {dd0, dd1, (double)d[2], (double)d[3]};
	double* bp[4] = {a.base.x, a.base.y, a.base.vx, a.base.vy};
	double* ap[4] = {a.acc.x, a.acc.y, a.acc.vx, a.acc.vy};
	double* sp[4] = {a.st.x, a.st.y, a.st.vx, a.st.vy};
	float* bq[4] = {a.base.rho_f, a.base.Sxx_f, a.base.Sxy_f, a.base.Syy_f};
	float* aq[4] = {a.acc.rho_f, a.acc.Sxx_f, a.acc.Sxy_f, a.acc.Syy_f};
	float* sq[4] = {a.st.rho_f, a.st.Sxx_f, a.st.Sxy_f, a.st.Syy_f};
	if (s < 3) {
		double dts = (s == 2 ? 1.0 : 0.5) * dt;
		double nv[4];  // the next stage's x, y, vx, vy
		float nf[4];   // and its rho - rho0, Sxx, Sxy, Syy
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ap[q][i] = (s == 0) ? dq[q] : ap[q][i] + 2 * dq[q];
			nv[q] = bp[q][i] + dq[q] * dts;
			sp[q][i] = nv[q];
			float dr = d[4 + q];
			aq[q][i] = (s == 0) ? dr : aq[q][i] + 2.f * dr;
			nf[q] = bq[q][i] + dr * (float)dts;
			sq[q][i] = nf[q];
		}
		if (a.write_recs)
			put_rec32(a, pr, i, reinterpret_cast<Rec32*>(a.rec_next) + k, nv[0], nv[1], nv[2], nv[3], nf[0], nf[1], nf[2],
			          nf[3]);
	} else {
		double w6 = dt * 1. / 6.;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			bp[q][i] = bp[q][i] + w6 * (ap[q][i] + dq[q]);
			bq[q][i] = bq[q][i] + (float)w6 * (aq[q][i] + d[4 + q]);
		}
		if (!(isfinite(bp[0][i]) && isfinite(bp[1][i]) && isfinite(bp[2][i]) && isfinite(bp[3][i]) &&
		      isfinite(bq[0][i])))
			fail_body(a.failed, st, ERR_NONFINITE, i, b);
	}
}

// The mixed pair pass with L threads per row (plain grid)
template <bool GOD, int L>
__global__ void __launch_bounds__(256, 3) k_pair_split(ULArgs a, const BodyParams* __restrict__ P,
                                                       const Geom* __restrict__ G, DevStatus* st) {
	const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t k = t / L;
	if (k >= a.n_total) return;  // a row's L lanes leave together (L divides the warp)
	pair32_row<GOD, L>(a, P, G, st, k, t % L);
}

// The pair kernels.  Plain form: one thread per cell-ordered row.  Persistent form
// (one launch per stage over all bodies): a fixed grid whose blocks take chunks of
// rows -- consecutive cell-ordered rows, so a chunk is a run of cells of one body --
// from an atomic counter until the rows run out; no block ever waits on another.
template <bool MIXED, bool GOD = false>
__global__ void __launch_bounds__(256, MIXED ? 3 : 1) k_pair(ULArgs a, const BodyParams* __restrict__ P, const Geom* __restrict__ G,
                                              DevStatus* st) {
	if (!a.persistent) {
		uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
		if (k >= a.n_total) return;
		if (MIXED) pair32_row<GOD>(a, P, G, st, k);
		else pair64_row(a, P, G, st, k);
		return;
	}
	__shared__ uint32_t s_chunk;
	const uint32_t rows = blockDim.x * a.chunk;
	for (;;) {
		if (threadIdx.x == 0) s_chunk = atomicAdd(a.work, 1u);
		__syncthreads();
		uint64_t base = (uint64_t)s_chunk * rows;
		__syncthreads();
		if (base >= a.n_total) break;
		for (uint32_t r = threadIdx.x; r < rows; r += blockDim.x) {
			uint64_t k = base + r;
			if (k < a.n_total) {
				if (MIXED) pair32_row<GOD>(a, P, G, st, (uint32_t)k);
				else pair64_row(a, P, G, st, (uint32_t)k);
			}
		}
	}
}

// Neighbour lists of the current grid (test/debug): pass 0 counts, pass 1 writes
// the rows of each list (as global rows) at offs[row].
__global__ void k_neighbors(ULArgs a, const Geom* __restrict__ G, uint32_t* counts, uint32_t* idx,
                            const uint64_t* offs, int pass) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.n_total) return;
	const Rec64* rec = reinterpret_cast<const Rec64*>(a.rec);
	const Rec64 ri = load_rec(rec + k);
	Geom g = G[a.rec_body[k]];
	uint32_t i = a.perm[k];
	int lo_i, hi_i, lo_j, hi_j;
	stencil(g, a.keys_sorted[k], lo_i, hi_i, lo_j, hi_j);
	const uint32_t tot = *a.total_cells;
	double hi = ri.h;
	double radius2 = __dmul_rn(__dmul_rn(__dmul_rn(hi, hi), 2.), 2.);
	double lim = __dadd_rn(radius2, a.nbh_eps);
	uint32_t cnt = 0;
	for (int ni = lo_i; ni < hi_i; ni++) {
		uint32_t c0 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)lo_j, tot);
		uint32_t c1 = min(g.cell_off + (uint32_t)ni * g.ny + (uint32_t)hi_j, tot);
		for (uint32_t kj = a.cell_start[c0]; kj < a.cell_start[c1]; kj++) {
			const Rec64 rj = load_rec(rec + kj);
			double xij = __dsub_rn(ri.x, rj.x);
			double yij = __dsub_rn(ri.y, rj.y);
			double r2 = __dadd_rn(__dmul_rn(xij, xij), __dmul_rn(yij, yij));
			if (r2 <= lim) {
				if (pass == 1) idx[offs[i] + cnt] = a.perm[kj];
				cnt++;
			}
		}
	}
	if (pass == 0) counts[i] = cnt;
}

inline unsigned grid1(uint32_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t build_grid(const ULArgs& a, bool mixed, cudaStream_t s) {
	DevStatus* st = reinterpret_cast<DevStatus*>(a.status);
	k_bbox_init<<<grid1(a.n_bodies, 128), 128, 0, s>>>(a.n_bodies, a.bbox);
	const mfk_host::StateSoA& sv = a.stage == 0 ? a.base : a.st;
	k_bbox<<<grid1(a.n_total, 256), 256, 0, s>>>(a.n_total, sv.x, sv.y, a.h, sv.vx, sv.vy, a.body_of, mixed ? 1 : 0,
	                                              a.bbox, a.failed);
	k_geom<<<1, 1024, 0, s>>>(a.n_bodies, a.bbox, a.params, mixed ? 1 : 0, a.geom, a.total_cells,
	                          a.cell_cap ? a.cell_cap : a.n_total + 1, st, a.failed);
	k_hash<<<grid1(a.n_total, 256), 256, 0, s>>>(a.n_total, sv.x, sv.y, a.body_of, a.geom, a.total_cells, a.keys,
	                                              a.perm_in, st, a.failed);
	size_t tmp = a.sort_tmp_bytes;
	cudaError_t e = cub::DeviceRadixSort::SortPairs(a.sort_tmp, tmp, a.keys, a.keys_sorted, a.perm_in, a.perm,
	                                                (int)a.n_total, 0, a.sort_bits, s);
	if (e != cudaSuccess) return e;
	k_cells<<<grid1(a.n_total + 1, 256), 256, 0, s>>>(a.n_total, a.keys_sorted, a.total_cells, a.cell_start);
	return cudaGetLastError();
}

}  // namespace

size_t ul_sort_tmp_bytes(uint32_t n, int bits) {
	size_t bytes = 0;
	cub::DeviceRadixSort::SortPairs(nullptr, bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
	                                (uint32_t*)nullptr, (int)n, 0, bits);
	return bytes;
}

size_t ul_rec_bytes(bool mixed) { return mixed ? sizeof(Rec32) : sizeof(Rec64); }

cudaError_t ul_stage(const ULArgs& a, bool mixed, cudaStream_t s) {
	if (a.n_total == 0) return cudaSuccess;
	DevStatus* st = reinterpret_cast<DevStatus*>(a.status);
	if (a.strict_grid || a.stage == 0) {
		cudaError_t e = build_grid(a, mixed, s);
		if (e != cudaSuccess) return e;
	}
	if (mixed) {
		if (!a.skip_gather) k_gather32<<<grid1(a.n_total, 256), 256, 0, s>>>(a, a.params);
	} else {
		k_gather64<<<grid1(a.n_total, 256), 256, 0, s>>>(a, a.params);
	}
	unsigned bs = a.block ? a.block : 128;
	unsigned grid = a.persistent ? a.grid : grid1(a.n_total, bs);
	if (a.persistent) {
		cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(uint32_t), s);
		if (e != cudaSuccess) return e;
	}
	if (a.ev_pair0) cudaEventRecord(a.ev_pair0, s);
	const bool god = a.flags & (A_GOD_CONT | A_GOD_MOM);
	if (mixed && !a.persistent && (a.split == 4 || a.split == 8)) {
		const unsigned g2 = grid1((uint64_t)a.n_total * a.split, bs);
		if (a.split == 4) {
			if (god) k_pair_split<true, 4><<<g2, bs, 0, s>>>(a, a.params, a.geom, st);
			else k_pair_split<false, 4><<<g2, bs, 0, s>>>(a, a.params, a.geom, st);
		} else {
			if (god) k_pair_split<true, 8><<<g2, bs, 0, s>>>(a, a.params, a.geom, st);
			else k_pair_split<false, 8><<<g2, bs, 0, s>>>(a, a.params, a.geom, st);
		}
	} else if (mixed && god) {
		k_pair<true, true><<<grid, bs, 0, s>>>(a, a.params, a.geom, st);
	} else if (mixed) {
		k_pair<true><<<grid, bs, 0, s>>>(a, a.params, a.geom, st);
	} else {
		k_pair<false><<<grid, bs, 0, s>>>(a, a.params, a.geom, st);
	}
	if (a.ev_pair1) cudaEventRecord(a.ev_pair1, s);
	return cudaGetLastError();
}

// left/right_bndry_fun_ul (tensile.cpp:44-66) on the particles after the RK4 combine
// (rk4.h:105): of what they set only the velocity outlives the step, since every
// derivative evaluation starts from zeroed rates
__global__ void k_ul_bc(uint32_t n_bc, const uint32_t* __restrict__ rows, const double* __restrict__ v, double* vx,
                        double* vy) {
	uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n_bc) return;
	uint32_t i = rows[k];
	vx[i] = v[k];
	vy[i] = 0.;
}

cudaError_t ul_bc(uint32_t n_bc, const uint32_t* rows, const double* v, double* vx, double* vy, cudaStream_t s) {
	k_ul_bc<<<grid1(n_bc, 128), 128, 0, s>>>(n_bc, rows, v, vx, vy);
	return cudaGetLastError();
}

cudaError_t ul_neighbors(const ULArgs& a, uint32_t* counts, uint32_t* idx, const uint64_t* offs, int pass,
                         cudaStream_t s) {
	if (a.n_total == 0) return cudaSuccess;
	if (pass == 0) {
		cudaError_t e = build_grid(a, false, s);
		if (e != cudaSuccess) return e;
		k_gather64<<<grid1(a.n_total, 256), 256, 0, s>>>(a, a.params);
	}
	k_neighbors<<<grid1(a.n_total, 128), 128, 0, s>>>(a, a.geom, counts, idx, offs, pass);
	return cudaGetLastError();
}

}  // namespace MF_NS
