// Penalty contact between bodies (contact_apply_body_to_boundary, contact.h:36-80),
// with the boundary refresh of body::update_boundary (body.h:153-166) and
// boundary::update_normals (boundary.h:50-76).
//
// The reference finds, for every slave particle, the nearest master boundary point
// with a kd-tree (kd_tree.cpp:61-101).  Here the master boundary (its points in tour
// order) is cut into tiles of 32 consecutive points with a bounding box each; a
// query first visits the tile whose box is nearest, then every other tile whose box
// can still hold a closer point.  Box tests run in FP32 on boxes grown by an
// absolute margin that covers FP32 rounding, so they never prune a tile that holds
// the nearest point; point distances are FP64 with the reference's operation order,
// so the nearest point is the kd-tree's.  Among exactly equal distances the lowest
// boundary index wins (the kd-tree keeps the first it meets in its traversal).
#include "mf_common.cuh"
#include "mf_kernels.h"

using namespace mfk;
using mfk_host::ContactArgs;

namespace MF_NS {
namespace {

inline unsigned grid1(uint64_t n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

constexpr float TILE_MARGIN = 1e-6f;  // metres; >> FP32 rounding of |coordinates| <= ~10 m

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

__device__ __forceinline__ float box_lb(float4 bb, float qx, float qy) {
	float dx = fmaxf(fmaxf(bb.x - qx, qx - bb.z), 0.f);
	float dy = fmaxf(fmaxf(bb.y - qy, qy - bb.w), 0.f);
	return dx * dx + dy * dy;
}

__device__ __forceinline__ void scan_tile(const ContactArgs& a, uint32_t t, double qx, double qy, double& best,
                                          uint32_t& arg) {
	for (uint32_t p = a.tile_first[t]; p < a.tile_end[t]; p++) {
		double4 q = a.bnd[p];
		double dx = qx - q.x, dy = qy - q.y;
		double dx2 = dx * dx, dy2 = dy * dy;
		double dist2 = dx2 + dy2;
		if (dist2 < best || (dist2 == best && p < arg)) {
			best = dist2;
			arg = p;
		}
	}
}

__global__ void __launch_bounds__(128) k_contact(ContactArgs a) {
	uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= a.n_slave) return;
	uint32_t row = a.slave_rows[r];
	uint32_t M = a.slave_master[r];
	uint32_t t0 = a.m_tile_off[M], t1 = t0 + a.m_tile_n[M];
	double qx = a.x[row], qy = a.y[row];
	float qxf = (float)qx, qyf = (float)qy;
	// nearest box first
	uint32_t tstar = t0;
	float lbstar = 3.4e38f;
	for (uint32_t t = t0; t < t1; t++) {
		float lb = box_lb(a.tile_bb[t], qxf, qyf);
		if (lb < lbstar) { lbstar = lb; tstar = t; }
	}
	double best = 1.7976931348623157e308;
	uint32_t arg = 0xffffffffu;
	if (t1 > t0) scan_tile(a, tstar, qx, qy, best, arg);
	for (uint32_t t = t0; t < t1; t++) {
		if (t == tstar) continue;
		float lb = box_lb(a.tile_bb[t], qxf, qyf);
		if (lb > __double2float_ru(best)) continue;
		scan_tile(a, t, qx, qy, best, arg);
	}
	double fx = 0., fy = 0.;
	if (arg != 0xffffffffu) {
		double4 cp = a.bnd[arg];
		double dx = qx - cp.x, dy = qy - cp.y;
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
