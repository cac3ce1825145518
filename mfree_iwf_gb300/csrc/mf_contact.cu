// Penalty contact between bodies (contact_apply_body_to_boundary, contact.h:36-80),
// with the boundary refresh of body::update_boundary (body.h:153-166) and
// boundary::update_normals (boundary.h:50-76).
//
// The reference finds, for every slave particle, the nearest master boundary point
// with a kd-tree (kd_tree.cpp:61-101).  Here the master boundary (its points in tour
// order) is cut into tiles of 32 consecutive points with an FP32 bounding box each,
// grown by an absolute margin that covers FP32 rounding.  A warp handles 32
// neighbouring slave particles: from the box around its queries it keeps only the
// tiles that can hold the nearest point of *some* query (lower bound <= the smallest
// upper bound over all tiles).  Each query then scans those tiles with its own
// box pruning, first in FP32 with float-float coordinate differences, then exactly in
// FP64 -- with the reference's operation order -- over the few points whose FP32
// distance is within 2e-5 (relative) of the FP32 minimum, a band that provably holds
// the exact minimum.  So the nearest point is the kd-tree's; among exactly equal
// distances the lowest boundary index wins (the kd-tree keeps the first it meets in
// its traversal).
#include "mf_common.cuh"
#include "mf_kernels.h"

using namespace mfk;
using mfk_host::ContactArgs;

namespace MF_NS {
namespace {

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

constexpr float TILE_MARGIN = 1e-6f;  // metres; > one FP32 ulp of |coordinates| < 16 m

__global__ void k_boundary(ContactArgs a) {
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= a.n_bnd) return;
	uint32_t b0 = a.bnd_start[p], nb = a.bnd_len[p];
	int i = (int)(p - b0);
	int left = i - 1, right = i + 1;
	if (left < 0) left = (int)nb - 1;
	if (right >= (int)nb) right = 0;
	uint32_t r = a.bnd_rows[p], rl = a.bnd_rows[b0 + left], rr = a.bnd_rows[b0 + right];
	double px = a.x[r], py = a.y[r];
	double tlx = a.x[rl] - px, tly = a.y[rl] - py;
	double trx = a.x[rr] - px, try_ = a.y[rr] - py;
	// normalize(v) = v * (1/sqrt(dot(v, v)))
	double ax = -tly, ay = tlx;
	double il = 1. / sqrt(ax * ax + ay * ay);
	double nlx = ax * il, nly = ay * il;
	double bx = try_, by = -trx;
	double ir = 1. / sqrt(bx * bx + by * by);
	double nrx = bx * ir, nry = by * ir;
	double nx = 0.5 * (nlx + nrx), ny = 0.5 * (nly + nry);
	a.bnd[p] = make_double4(px, py, nx, ny);
	FF fx = ff_split(px), fy = ff_split(py);
	a.bnd_ff[p] = make_float4(fx.hi, fx.lo, fy.hi, fy.lo);
}

__global__ void k_tiles(ContactArgs a) {
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= a.n_tiles) return;
	uint32_t p0 = a.tile_first[t], p1 = a.tile_end[t];
	float mnx = 3e38f, mny = 3e38f, mxx = -3e38f, mxy = -3e38f;
	for (uint32_t p = p0; p < p1; p++) {
		double4 q = a.bnd[p];
		mnx = fminf(mnx, __double2float_rd(q.x));
		mny = fminf(mny, __double2float_rd(q.y));
		mxx = fmaxf(mxx, __double2float_ru(q.x));
		mxy = fmaxf(mxy, __double2float_ru(q.y));
	}
	a.tile_bb[t] = make_float4(mnx - TILE_MARGIN, mny - TILE_MARGIN, mxx + TILE_MARGIN, mxy + TILE_MARGIN);
}

// squared distance bounds between a query box (x0, y0, x1, y1) and a tile box
__device__ __forceinline__ float box_lb(float4 bb, float x0, float y0, float x1, float y1) {
	float dx = fmaxf(fmaxf(bb.x - x1, x0 - bb.z), 0.f);
	float dy = fmaxf(fmaxf(bb.y - y1, y0 - bb.w), 0.f);
	return dx * dx + dy * dy;
}
__device__ __forceinline__ float box_ub(float4 bb, float x0, float y0, float x1, float y1) {
	float dx = fmaxf(fabsf(bb.z - x0), fabsf(x1 - bb.x));
	float dy = fmaxf(fabsf(bb.w - y0), fabsf(y1 - bb.y));
	return dx * dx + dy * dy;
}

struct Query {
	float xf, yf;       // FP32 coordinates (box tests)
	FF x, y;            // float-float (FP32 distances)
	double xd, yd;      // FP64 (exact distances)
};

__device__ __forceinline__ float ff_dist2(const Query& q, float4 p) {
	float dx = (q.x.hi - p.x) + (q.x.lo - p.y);
	float dy = (q.y.hi - p.z) + (q.y.lo - p.w);
	return dx * dx + dy * dy;
}

// FP32 pass over one tile: the smallest FP32 distance
__device__ __forceinline__ void scan_f32(const ContactArgs& a, uint32_t t, const Query& q, float& best_f) {
	for (uint32_t p = a.tile_first[t]; p < a.tile_end[t]; p++) best_f = fminf(best_f, ff_dist2(q, a.bnd_ff[p]));
}
// exact pass over one tile: FP64 distances (kd_tree.cpp:79-88 order) of the points in the band
__device__ __forceinline__ void scan_exact(const ContactArgs& a, uint32_t t, const Query& q, float thr, double& best,
                                           uint32_t& arg) {
	for (uint32_t p = a.tile_first[t]; p < a.tile_end[t]; p++) {
		if (ff_dist2(q, a.bnd_ff[p]) > thr) continue;
		double4 c = a.bnd[p];
		double dx = q.xd - c.x, dy = q.yd - c.y;
		double dx2 = dx * dx, dy2 = dy * dy;
		double dist2 = dx2 + dy2;
		if (dist2 < best || (dist2 == best && p < arg)) {
			best = dist2;
			arg = p;
		}
	}
}

__global__ void __launch_bounds__(128) k_contact(ContactArgs a) {
	const unsigned FULL = 0xffffffffu;
	uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	bool valid = r < a.n_slave;
	unsigned vmask = __ballot_sync(FULL, valid);
	if (!vmask) return;  // the whole warp is past the end
	uint32_t lane = threadIdx.x & 31;
	uint32_t row = valid ? a.slave_rows[r] : 0u;
	uint32_t M = valid ? a.slave_master[r] : 0u;
	uint32_t M0 = __shfl_sync(FULL, M, __ffs(vmask) - 1);
	if (!valid) M = M0;
	bool uniform = __all_sync(FULL, M == M0);
	Query q;
	q.xd = valid ? a.x[row] : 0.;
	q.yd = valid ? a.y[row] : 0.;
	// integer-only splits (conversions from FP64 would occupy the narrow FP64 pipe for
	// every query); the box tests take hi, within one FP32 ulp of the coordinate, which
	// TILE_MARGIN covers
	q.x = ff_split_bits(q.xd);
	q.y = ff_split_bits(q.yd);
	q.xf = q.x.hi;
	q.yf = q.y.hi;
	uint32_t t0 = a.m_tile_off[M], nt = a.m_tile_n[M];
	float best_f = 3.4e38f;
	double best = 1.7976931348623157e308;
	uint32_t arg = 0xffffffffu;
	if (uniform) {
		// the warp's query box
		float x0 = valid ? q.xf : 3.4e38f, y0 = valid ? q.yf : 3.4e38f;
		float x1 = valid ? q.xf : -3.4e38f, y1 = valid ? q.yf : -3.4e38f;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			x0 = fminf(x0, __shfl_xor_sync(FULL, x0, o));
			y0 = fminf(y0, __shfl_xor_sync(FULL, y0, o));
			x1 = fmaxf(x1, __shfl_xor_sync(FULL, x1, o));
			y1 = fmaxf(y1, __shfl_xor_sync(FULL, y1, o));
		}
		// an upper bound of every query's nearest squared distance: the farthest a query of
		// the box can be from some tile's first point (a tile box's farthest corner would
		// add up to a tile's length, and with it every tile within that much more)
		float ubmin = 3.4e38f;
		for (uint32_t t = lane; t < nt; t += 32) {
			const float4 p = a.bnd_ff[a.tile_first[t0 + t]];  // hi parts: within TILE_MARGIN of the point
			const float4 pb = make_float4(p.x - TILE_MARGIN, p.z - TILE_MARGIN, p.x + TILE_MARGIN, p.z + TILE_MARGIN);
			ubmin = fminf(ubmin, box_ub(pb, x0, y0, x1, y1));
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) ubmin = fminf(ubmin, __shfl_xor_sync(FULL, ubmin, o));
		float cut = ubmin * (1.f + 1e-5f);
		best_f = cut;  // an upper bound of every query's nearest squared distance
		// FP32 pass over the warp's candidate tiles
		for (uint32_t c0 = 0; c0 < nt; c0 += 32) {
			bool cand = c0 + lane < nt && box_lb(a.tile_bb[t0 + c0 + lane], x0, y0, x1, y1) <= cut;
			unsigned m = __ballot_sync(FULL, cand);
			while (m) {
				uint32_t t = t0 + c0 + (__ffs(m) - 1);
				m &= m - 1;
				if (valid && box_lb(a.tile_bb[t], q.xf, q.yf, q.xf, q.yf) <= best_f) scan_f32(a, t, q, best_f);
			}
		}
		// exact pass: every tile that can hold a point within the band of some query
		float thr = best_f * (1.f + 2e-5f) + 1e-37f;
		float thr_w = valid ? thr : 0.f;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) thr_w = fmaxf(thr_w, __shfl_xor_sync(FULL, thr_w, o));
		for (uint32_t c0 = 0; c0 < nt; c0 += 32) {
			bool cand = c0 + lane < nt && box_lb(a.tile_bb[t0 + c0 + lane], x0, y0, x1, y1) <= thr_w;
			unsigned m = __ballot_sync(FULL, cand);
			while (m) {
				uint32_t t = t0 + c0 + (__ffs(m) - 1);
				m &= m - 1;
				if (valid && box_lb(a.tile_bb[t], q.xf, q.yf, q.xf, q.yf) <= thr) scan_exact(a, t, q, thr, best, arg);
			}
		}
	} else if (valid) {
		// mixed masters in this warp (the seam between two slave bodies): query alone
		for (uint32_t t = 0; t < nt; t++)
			if (box_lb(a.tile_bb[t0 + t], q.xf, q.yf, q.xf, q.yf) <= best_f) scan_f32(a, t0 + t, q, best_f);
		float thr = best_f * (1.f + 2e-5f) + 1e-37f;
		for (uint32_t t = 0; t < nt; t++)
			if (box_lb(a.tile_bb[t0 + t], q.xf, q.yf, q.xf, q.yf) <= thr) scan_exact(a, t0 + t, q, thr, best, arg);
	}
	if (!valid) return;
	if (arg == 0xffffffffu)  // cannot happen with the bounds above; kept as a full exact fallback
		for (uint32_t t = 0; t < nt; t++) scan_exact(a, t0 + t, q, 3.4e38f, best, arg);
	double fx = 0., fy = 0.;
	if (arg != 0xffffffffu) {
		double4 cp = a.bnd[arg];
		double dx = q.xd - cp.x, dy = q.yd - cp.y;
		double pdotn = dx * cp.z + dy * cp.w;
		if (pdotn <= 0.) {
			double gN_nx = cp.z * pdotn, gN_ny = cp.w * pdotn;
			double ms = a.m[row];
			double dt = a.dt[r];
			double dt2 = dt * dt;
			const double alpha = 0.1;
			fx = -(ms * gN_nx / dt2 * alpha);
			fy = -(ms * gN_ny / dt2 * alpha);
		}
	}
	a.fcx[row] = fx;
	a.fcy[row] = fy;
}

}  // namespace

cudaError_t contact_step(const ContactArgs& a, cudaStream_t s) {
	if (a.n_bnd == 0) return cudaSuccess;
	k_boundary<<<grid1(a.n_bnd, 128), 128, 0, s>>>(a);
	k_tiles<<<grid1(a.n_tiles, 128), 128, 0, s>>>(a);
	if (a.n_slave) k_contact<<<grid1(a.n_slave, 128), 128, 0, s>>>(a);
	return cudaGetLastError();
}

}  // namespace MF_NS
