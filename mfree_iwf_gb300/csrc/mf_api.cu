// Host side of the C ABI (include/mfree_gb300.h): contexts, bodies, action-list
// validation against the fused pipelines, device memory, and the step loop of the
// reference driver (mfree_iwf.cpp:84-97) expressed as stream-ordered launches.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mfree_gb300.h"
#include "mf_kernels.h"

using namespace mfk_host;

namespace {

const uint32_t REF_MAX_NBH = 200;  // particle.h:31

// Per-body reductions of the current state, one row per step into a device ring of
// `cap` rows: [mean vx, mean vy, max von Mises stress, sum |fc|] per body.  sigma =
// S - p I with p from the EOS (material.h:37-44); plane von Mises
// sqrt(sxx^2 - sxx syy + syy^2 + 3 sxy^2).  One block per body; the row index comes
// from a device counter so the kernel can live inside a captured step graph.
__global__ void k_monitor(uint32_t nb, const BodyParams* __restrict__ P, const double* __restrict__ vx,
                          const double* __restrict__ vy, const double* __restrict__ rho, const float* __restrict__ rho_f,
                          const double* __restrict__ Sxx, const double* __restrict__ Sxy, const double* __restrict__ Syy,
                          const float* __restrict__ Sxx_f, const float* __restrict__ Sxy_f, const float* __restrict__ Syy_f,
                          const double* __restrict__ fcx, const double* __restrict__ fcy, uint32_t eos, float* out,
                          uint32_t* counter, uint32_t cap) {
	uint32_t b = blockIdx.x;
	if (b >= nb) return;
	const BodyParams& pr = P[b];
	double svx = 0., svy = 0., vm = 0., fc = 0.;
	for (uint32_t k = threadIdx.x; k < pr.n; k += blockDim.x) {
		uint32_t i = pr.off + k;
		svx += vx[i];
		svy += vy[i];
		double r = rho ? rho[i] : (double)rho_f[i] + pr.rho0;
		double p = eos ? pr.c0sq * (r - pr.rho0) : 0.;
		double sxx = (Sxx ? Sxx[i] : (double)Sxx_f[i]) - p;
		double syy = (Syy ? Syy[i] : (double)Syy_f[i]) - p;
		double sxy = Sxy ? Sxy[i] : (double)Sxy_f[i];
		vm = fmax(vm, sqrt(fmax(sxx * sxx - sxx * syy + syy * syy + 3. * sxy * sxy, 0.)));
		fc += sqrt(fcx[i] * fcx[i] + fcy[i] * fcy[i]);
	}
	__shared__ double s0[256], s1[256], s2[256], s3[256];
	s0[threadIdx.x] = svx; s1[threadIdx.x] = svy; s2[threadIdx.x] = vm; s3[threadIdx.x] = fc;
	__syncthreads();
	for (uint32_t o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			s0[threadIdx.x] += s0[threadIdx.x + o];
			s1[threadIdx.x] += s1[threadIdx.x + o];
			s2[threadIdx.x] = fmax(s2[threadIdx.x], s2[threadIdx.x + o]);
			s3[threadIdx.x] += s3[threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		uint32_t row = *counter % cap;
		float* o = out + ((size_t)row * nb + b) * 4;
		o[0] = (float)(s0[0] / pr.n);
		o[1] = (float)(s1[0] / pr.n);
		o[2] = (float)s2[0];
		o[3] = (float)s3[0];
	}
}
__global__ void k_monitor_tick(uint32_t* counter) { *counter += 1; }

// FP64 <-> FP32 state fields; the mixed form keeps the density as its deviation from
// rho0 (`off`), which resolves per-step density changes far below rho0's FP32 ulp.
__global__ void k_f64_to_f32(uint32_t n, const double* __restrict__ a, float* __restrict__ b, double off) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = (float)(a[i] - off);
}
__global__ void k_f32_to_f64(uint32_t n, const float* __restrict__ a, double* __restrict__ b, double off) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = off + (double)a[i];
}
// the same over all bodies' rows, the density offset being each row's body's rho0
__global__ void k_f64_to_f32_rows(uint32_t n, const double* __restrict__ a, float* __restrict__ b,
                                  const uint32_t* __restrict__ body_of, const BodyParams* __restrict__ P, int rho) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = (float)(a[i] - (rho ? P[body_of[i]].rho0 : 0.));
}
__global__ void k_f32_to_f64_rows(uint32_t n, const float* __restrict__ a, double* __restrict__ b,
                                  const uint32_t* __restrict__ body_of, const BodyParams* __restrict__ P, int rho) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) b[i] = (rho ? P[body_of[i]].rho0 : 0.) + (double)a[i];
}

// All-body state transfers in one pass when the host arrays are device-accessible
// (pinned and mapped, or system memory the GPU reaches through the CPU's page tables,
// as on a C2C-coupled Grace host): each row's fields cross the link once, coalesced,
// with the FP32 conversion of the mixed form and the copy into the TL stage set fused.
// Same values as the copy-and-convert path.
struct StateIO {
	const double* src[8];  // set: host x y vx vy rho Sxx Sxy Syy (null: field untouched)
	double* dst[10];       // get: host x y vx vy rho Sxx Sxy Syy fcx fcy (null: not read)
	double* sd0[8];        // device FP64 state (null where the mixed form keeps FP32)
	double* sd2[8];        // device TL stage-0 copy (null: none)
	float* sf0[4];         // mixed: rho - rho0, Sxx, Sxy, Syy
	float* sf2[4];
	const double *fcx, *fcy;
};
__global__ void k_set_state_io(uint32_t n, StateIO io, const uint32_t* __restrict__ body_of,
                               const BodyParams* __restrict__ P) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
#pragma unroll
	for (int q = 0; q < 8; q++) {
		if (!io.src[q]) continue;
		double v = io.src[q][i];
		if (q >= 4 && io.sf0[q - 4]) {
			float f = (float)(v - (q == 4 ? P[body_of[i]].rho0 : 0.));
			io.sf0[q - 4][i] = f;
			if (io.sf2[q - 4]) io.sf2[q - 4][i] = f;
		} else {
			io.sd0[q][i] = v;
			if (io.sd2[q]) io.sd2[q][i] = v;
		}
	}
}
__global__ void k_get_state_io(uint32_t n, StateIO io, const uint32_t* __restrict__ body_of,
                               const BodyParams* __restrict__ P) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
#pragma unroll
	for (int q = 0; q < 8; q++) {
		if (!io.dst[q]) continue;
		if (q >= 4 && io.sf0[q - 4]) io.dst[q][i] = (q == 4 ? P[body_of[i]].rho0 : 0.) + (double)io.sf0[q - 4][i];
		else io.dst[q][i] = io.sd0[q][i];
	}
	if (io.dst[8]) io.dst[8][i] = io.fcx[i];
	if (io.dst[9]) io.dst[9][i] = io.fcy[i];
}

struct HostBC {
	int32_t kind;
	double v;
	std::vector<uint32_t> idx;
};

struct HostBody {
	uint32_t off = 0, n = 0;
	mf_sim_data sd{};
	double dt = 0., time = 0.;
	int32_t group = 0;
	std::vector<int32_t> actions;
	std::vector<uint32_t> hull;
	std::vector<HostBC> bcs;
	std::vector<double> in[13];  // x y X Y m rho h qw vx vy Sxx Sxy Syy
	uint32_t ex = 0, ey = 0;     // TL_WEAK: element_map_rectangle(ex, ey), 2x2 Gauss points
	std::vector<uint32_t> quads;  // TL_WEAK: explicit element map (ll lr tr tl, body-local), mf_set_elements
	uint32_t order = 2;
	int32_t shape = MF_SHAPE_RKPM;
	double gp_h = 0., gp_rho = 0.;
	std::vector<double> gpt[4];  // TL_WEAK: given Gauss-point x, y, h, rho (mf_set_gauss_points)
	uint32_t n_sp = 0;           // UL_WEAK: stress points (mf_set_stress_points), same fields as `in`
	std::vector<double> sp[13];
};

template <class T>
struct DevBuf {
	T* p = nullptr;
	size_t n = 0;
	cudaError_t alloc(size_t count) {
		n = count;
		return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
	}
	void free() {
		if (p) cudaFree(p);
		p = nullptr;
	}
};

struct Timing {
	bool on = false;
	std::vector<cudaEvent_t> pool;
	std::vector<std::pair<int, int>> used;  // (kind, pool index of start)
	double ms[8] = {0};
	uint64_t launches[8] = {0};
	uint64_t rows[8] = {0};
};

// Launch shape of the hot kernels, chosen by mf_autotune.
struct Tune {
	uint32_t ul_block = 128, ul_persistent = 0, ul_chunk = 1, tl_block = 128;
	uint32_t ul_split = 1;  // mixed UL, plain grid: threads per row of the pair pass
	uint32_t tl_tiled = 0;  // mixed TL: the halo-tile passes (built at set-up when requested)
	uint32_t tl_runs = 1;   // mixed TL: the run-walk passes (gradients recomputed on chip)
	uint32_t tl_unroll = 1; // run walk: 1 or 2 pairs per iteration, 3: pass B at 64 registers, 4: and pass A at
	                        // 48 (same results)
};
std::mutex g_tune_mutex;
std::map<std::string, Tune> g_tune_cache;

}  // namespace

struct mf_ctx {
	mf_config cfg{};
	cudaStream_t stream = nullptr;
	std::string err;
	std::vector<HostBody> bodies;
	bool ready = false;
	uint32_t n_total = 0;
	uint32_t flags = 0;
	bool mixed = false, strict = false;
	bool uw_mixed = false;  // weak UL, mixed form: FP32 ellipse and moments, FP32 / float-float pass sums
	uint64_t launches = 0;
	Timing timing;

	DevStatusH* d_status = nullptr;
	DevStatusH* h_status = nullptr;

	// common per-row arrays
	DevBuf<uint32_t> body_of;
	DevBuf<double> m, h, qw0, fcx, fcy, X, Y;
	DevBuf<double> sd[4][8];   // base, acc, stage, second stage (TL ping-pong): x y vx vy rho Sxx Sxy Syy
	DevBuf<float> sf[4][4];    // mixed form: rho Sxx Sxy Syy
	DevBuf<BodyParams> params;
	std::vector<BodyParams> h_params;

	// UL
	DevBuf<Geom> geom;
	DevBuf<unsigned long long> bbox;
	DevBuf<uint32_t> total_cells, keys, keys_sorted, perm_in, perm, cell_start, rec_body;
	DevBuf<unsigned char> rec, sort_tmp;
	DevBuf<unsigned char> rec2;  // mixed UL: the second record buffer (stages alternate between the two)
	int sort_bits = 1;
	uint32_t cell_cap = 0;

	// TL: fixed neighbour lists (CSR from the set-up, kept for mf_get_neighbors, and the
	// sliced-ELL copy the stage kernels read) with corrected gradients, per-stage scratch
	DevBuf<uint32_t> nbr_off, nbr, bc_rows, sl_off, snbr;
	DevBuf<uint16_t> scnt;
	DevBuf<double> wx64, wy64, P64, dA64, c64, bc_v;
	DevBuf<double2> sw64;
	DevBuf<float2> sw32, swA32;
	// mixed TL halo tiles (TLArgs::t_*)
	DevBuf<uint32_t> tt_rows, tt_halo_off, tt_halo, tt_sl;
	DevBuf<uint16_t> tt_cnt, tt_loc;
	DevBuf<float2> tt_sw, tt_swA;
	uint32_t tt_n_tiles = 0, tt_halo_max = 0, tt_ent_max = 0;
	bool tt_ok = false;
	// mixed TL run walk (TLArgs::r_sl, r_cnt, runs, XF, G)
	DevBuf<uint32_t> rw_sl, rw_runs;
	DevBuf<uint16_t> rw_cnt;
	DevBuf<float4> rw_XF, rw_G;
	bool rw_ok = false;
	uint64_t rw_words = 0;
	DevBuf<float> qw32, m32, h32;
	DevBuf<float4> recA, recB, dA32;
	DevBuf<float4> recB2;             // mixed TL: records ping-pong between recB and recB2 by stage parity
	DevBuf<double> sW64, R64, av64;   // corotational: W per pair (sliced ELL), rotation per row;
	                                  // corotational / potential: the viscosity records
	// corotational / potential, mixed form (TLArgs::cm_*)
	DevBuf<float2> cm_sw, cm_swA, cm_sX, cm_swji;
	DevBuf<float> cm_sW;
	DevBuf<float4> cm_U, cm_X, cm_V, cm_P, cm_R, cm_H;
	bool tl_recs_valid = false;       // the stage-0 records match the state (pass B keeps them current)
	// UL: per-body failure words (ERR_* bits); used by the kernels when mask_failed is set
	DevBuf<uint32_t> failed;
	bool mask_failed = false;
	uint32_t n_bc = 0;

	// TL_WEAK: Gauss points and the three list sets (sliced ELL)
	uint32_t n_g = 0;
	uint64_t g_entries = 0, t_entries = 0;  // TL_WEAK: list entries of the Gauss points and of the particles' transposed lists
	DevBuf<uint32_t> gp_body, g_sl, g_snbr, t_sl, t_snbr, p_sl, p_snbr;
	DevBuf<uint16_t> g_cnt, t_cnt, p_cnt;
	DevBuf<double> gp_x, gp_y, gp_qw, gp_hh, gp_ux, gp_uy, gsd[3][4], gP64;
	DevBuf<float> gsf[3][4];
	DevBuf<float4> gP32, wpack;
	DevBuf<double2> g_w64, t_w64, p_w64;
	DevBuf<float2> g_w32, t_w32, p_w32;
	bool do_smooth = false;

	// UL_WEAK: stress points (state sets as the particles: base, accumulator, two stage
	// sets), fixed candidate lists, per-evaluation ellipse masks and shape functions
	DevBuf<uint32_t> uw_gbody, uw_pc_off, uw_pc_nbr, uw_gc_off, uw_gc_nbr, uw_tp_off, uw_tp_gp, uw_tp_slot, uw_bc_of;
	DevBuf<uint32_t> uw_pc_cnt, uw_gc_cnt, uw_tp_cnt;  // entries per row; *_off hold the rows' first slots
	uint32_t uw_pc_stride = 1, uw_gc_stride = 1;
	DevBuf<uint8_t> uw_pmask, uw_gmask;
	DevBuf<double> uw_pw, uw_pwx, uw_pwy, uw_gw, uw_gwx, uw_gwy, uw_gsig, uw_ph, uw_gh, uw_qwp, uw_qws, uw_gm, uw_gqw;
	DevBuf<double> uw_g[4][6];  // x y rho Sxx Sxy Syy
	DevBuf<float> uw_ff, uw_vol;  // mixed form: the stage's float-float positions, FP32 volumes
	DevBuf<float> uw_vff, uw_qw32, uw_qwlo, uw_gsig32;  // and velocities, weights, stress points' gsig
	DevBuf<uint32_t> uw_quads;  // element maps (global ll lr tr tl) when a gauss_int replaces the ellipse
	uint32_t uw_order = 0, uw_nelem = 0;

	// host <-> device state transfers: FP64 staging for the fields stored as FP32
	DevBuf<double> staging;

	// state dumps (VTK, checkpoints): device snapshot, then copy-out and file write on a
	// host thread with its own stream while the simulation goes on
	DevBuf<unsigned char> io_dev;
	unsigned char* io_host = nullptr;
	size_t io_host_bytes = 0;
	cudaStream_t io_stream = nullptr;
	// stream-ordered state transfers (mf_*_state_all_async): a device->host and a
	// host->device copy stream, FP64 staging of all fields, one event per field
	cudaStream_t xs_d2h = nullptr, xs_h2d = nullptr;
	cudaEvent_t xe_main = nullptr, xe_d2h[10] = {};
	cudaEvent_t xe_conv[10] = {}, xe_in[8] = {};  // per field: converted into the staging / copied in
	bool xe_pending[10] = {};  // a get of field q was queued since the last synchronize
	DevBuf<double> x_out, x_in;
	cudaEvent_t io_ready = nullptr;
	std::thread io_thread;
	mf_status io_status = MF_OK;
	std::string io_err;

	// per-step monitor (mf_set_monitor)
	uint32_t mon_cap = 0;
	DevBuf<float> mon;
	DevBuf<uint32_t> mon_counter;

	// launch shapes, persistent-kernel work counter, captured step graph
	Tune tune;
	int sm_count = 0;
	DevBuf<uint32_t> work;
	// [0]: a step; [1]: a step that starts with the pending contact query (contact_pending)
	cudaGraph_t graph[2] = {nullptr, nullptr};
	cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
	uint64_t graph_launches[2] = {0, 0};
	bool graph_deferred = false;  // contact_deferred() when the graphs were captured

	// contact
	bool contact_on = false;
	// mixed TL: the contact query of the positions a step ends with runs at the start of
	// the next step, beside stage 0's pass A on a side stream (contact_overlap, default on)
	bool contact_overlap = true, contact_pending = false;
	bool async_steps = false;  // mf_step queues only; the status is read at the next synchronization
	cudaStream_t side = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	DevBuf<uint32_t> bnd_rows, bnd_start, bnd_len, tile_first, tile_end, slave_rows, slave_master, m_tile_off, m_tile_n;
	DevBuf<double4> bnd;
	DevBuf<float4> tile_bb, bnd_ff;
	DevBuf<double> slave_dt;
	uint32_t n_bnd = 0, n_tiles = 0, n_slave = 0;

	~mf_ctx();
};

namespace {

mf_status fail(mf_ctx* c, mf_status s, const char* fmt, ...) {
	if (c) {
		char buf[512];
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(buf, sizeof buf, fmt, ap);
		va_end(ap);
		c->err = buf;
	}
	return s;
}

mf_status cuda_fail(mf_ctx* c, cudaError_t e, const char* where) {
	return fail(c, MF_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define CK(call)                                            \
	do {                                                    \
		cudaError_t e_ = (call);                            \
		if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
	} while (0)

inline uint32_t abit(int a) { return 1u << a; }

mf_status validate_tl(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags);
mf_status validate_corot(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags);
mf_status validate_potential(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags);
mf_status validate_ulweak(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags);
mf_status uw_setup(mf_ctx* c);
mf_status uw_step(mf_ctx* c);
mf_status tl_setup(mf_ctx* c);
mf_status weak_setup(mf_ctx* c);
mf_status validate_weak(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags);
mf_status contact_setup(mf_ctx* c);
mf_status upload_bcs(mf_ctx* c);

// UL pipeline: a subsequence, in this order, of the union of the reference's
// rings_monaghan list (rings.cpp:86-96) and rings_godunov list (rings.cpp:154-160),
// with the data dependencies present.  The Godunov actions take the flag bits
// FLAG_GODUNOV_* and run in the FP64 forms.
mf_status validate_ul(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS, MF_MATERIAL_EOS, MF_CORRECTORS_MGHN_ARTIFICIAL_STRESS,
	                            MF_DERIVE_STRESS_MONAGHAN, MF_DERIVE_VELOCITY, MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
	                            MF_CORRECTORS_XSPH, MF_MATERIAL_STRESS_RATE_JAUMANN, MF_CONTMECH_CONTINUITY,
	                            MF_GODUNOV_CONTINUITY, MF_GODUNOV_MOMENTUM, MF_CONTMECH_MOMENTUM_UL, MF_CONTMECH_ADVECTION};
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not an updated-Lagrangian action or out of the fused UL order", a);
		pos++;
		flags |= a == MF_GODUNOV_CONTINUITY ? FLAG_GODUNOV_CONTINUITY
		         : a == MF_GODUNOV_MOMENTUM ? FLAG_GODUNOV_MOMENTUM
		                                    : abit(a);
	}
	if ((flags & abit(MF_CONTMECH_MOMENTUM_UL)) && !(flags & abit(MF_DERIVE_STRESS_MONAGHAN)))
		return fail(c, MF_ERR_PIPELINE, "contmech_momentum_ul needs derive_stress_monaghan before it");
	if ((flags & (abit(MF_MATERIAL_STRESS_RATE_JAUMANN) | abit(MF_CONTMECH_CONTINUITY))) &&
	    !(flags & abit(MF_DERIVE_VELOCITY)))
		return fail(c, MF_ERR_PIPELINE, "Jaumann rate / continuity need derive_velocity before them");
	const uint32_t god = FLAG_GODUNOV_CONTINUITY | FLAG_GODUNOV_MOMENTUM;
	if (flags & god) {
		if ((flags & FLAG_GODUNOV_CONTINUITY) && (flags & abit(MF_CONTMECH_CONTINUITY)))
			return fail(c, MF_ERR_PIPELINE, "godunov_continuity and contmech_continuity both set the density rate");
		if ((flags & FLAG_GODUNOV_MOMENTUM) && (flags & abit(MF_CONTMECH_MOMENTUM_UL)))
			return fail(c, MF_ERR_PIPELINE, "godunov_momentum and contmech_momentum_ul both add the stress forces");
		if (flags & abit(MF_CORRECTORS_MGHN_ARTIFICIAL_STRESS))
			return fail(c, MF_ERR_PIPELINE, "the Godunov actions do not combine with the artificial stress");
	}
	return MF_OK;
}

BodyParams make_params(const HostBody& b) {
	BodyParams p{};
	double nu = b.sd.nu, E = b.sd.E, rho0 = b.sd.rho0;
	// physical_constants, simulation_data.cpp:32-47
	double G = E / (2. * (1. + nu));
	double K = 2.0 * G * (1 + nu) / (3 * (1 - 2 * nu));
	double c0 = sqrt(K / rho0);
	p.K = K; p.G = G; p.rho0 = rho0; p.c0sq = c0 * c0;
	p.E = E; p.nu = nu; p.D = E / (1 - nu * nu);
	p.wdeltap = b.sd.mghn_wdeltap; p.corr_exp = b.sd.mghn_corr_exp; p.mghn_eps = b.sd.mghn_eps;
	p.alpha = b.sd.artvisc_alpha; p.beta = b.sd.artvisc_beta; p.eta = b.sd.artvisc_eta; p.xsph_eps = b.sd.xsph_eps;
	p.dt = b.dt; p.time = b.time;
	p.off = b.off; p.n = b.n;
	p.fK = (float)p.K; p.fG = (float)p.G; p.frho0 = (float)p.rho0; p.fc0sq = (float)p.c0sq; p.fD = (float)p.D;
	p.fnu = (float)p.nu; p.falpha = (float)p.alpha; p.fbeta = (float)p.beta; p.feta2 = (float)(p.eta * p.eta);
	p.fdt = (float)p.dt;
	p.fwdp1 = p.wdeltap > 0 ? (float)(1.0 / p.wdeltap) : 0.f;
	p.fcorr_exp = (float)p.corr_exp; p.fxsph_eps = (float)p.xsph_eps; p.fmghn_eps = (float)p.mghn_eps;
	return p;
}

ULArgs ul_args(mf_ctx* c, uint32_t stage) {
	ULArgs a{};
	a.n_total = c->n_total;
	a.n_bodies = (uint32_t)c->bodies.size();
	a.stage = stage;
	a.flags = c->flags;
	a.max_nbh = c->cfg.max_nbh;
	a.strict_grid = c->mixed ? 0u : 1u;
	a.nbh_eps = c->cfg.nbh_eps;
	a.params = c->params.p;
	a.geom = c->geom.p;
	a.bbox = c->bbox.p;
	a.total_cells = c->total_cells.p;
	a.body_of = c->body_of.p;
	a.m = c->m.p; a.h = c->h.p; a.qw0 = c->qw0.p; a.fcx = c->fcx.p; a.fcy = c->fcy.p;
	StateSoA* s[3] = {&a.base, &a.acc, &a.st};
	for (int k = 0; k < 3; k++) {
		double** d[8] = {&s[k]->x, &s[k]->y, &s[k]->vx, &s[k]->vy, &s[k]->rho, &s[k]->Sxx, &s[k]->Sxy, &s[k]->Syy};
		for (int q = 0; q < 8; q++) *d[q] = c->sd[k][q].p;
		s[k]->rho_f = c->sf[k][0].p; s[k]->Sxx_f = c->sf[k][1].p; s[k]->Sxy_f = c->sf[k][2].p; s[k]->Syy_f = c->sf[k][3].p;
	}
	a.keys = c->keys.p; a.keys_sorted = c->keys_sorted.p; a.perm_in = c->perm_in.p; a.perm = c->perm.p;
	a.cell_start = c->cell_start.p;
	a.rec = c->rec.p;
	a.rec_body = c->rec_body.p;
	if (c->mixed && c->rec2.p && !a.strict_grid) {
		// the cell order holds for the whole step: stage s reads record buffer s % 2, and
		// its pair pass (stages 0-2) writes the next stage's records into the other one
		unsigned char* rb[2] = {c->rec.p, c->rec2.p};
		a.rec = rb[stage & 1];
		a.rec_next = rb[(stage + 1) & 1];
		a.write_recs = stage < 3 ? 1u : 0u;
		a.skip_gather = stage > 0 ? 1u : 0u;
	}
	a.sort_tmp = c->sort_tmp.p;
	a.sort_tmp_bytes = c->sort_tmp.n;
	a.sort_bits = c->sort_bits;
	a.cell_cap = c->cell_cap;
	a.status = c->d_status;
	a.block = c->tune.ul_block;
	a.persistent = c->tune.ul_persistent;
	a.chunk = c->tune.ul_chunk;
	a.split = c->tune.ul_split;
	a.grid = (uint32_t)std::max(1, c->sm_count) * (2048u / c->tune.ul_block);
	a.work = c->work.p;
	a.failed = c->mask_failed ? c->failed.p : nullptr;
	return a;
}

// ---------------------------------------------------------------- timing
cudaEvent_t timing_begin(mf_ctx* c, int kind, int& slot) {
	slot = -1;
	if (!c->timing.on) return nullptr;
	Timing& t = c->timing;
	if (t.used.size() * 2 + 2 > t.pool.size()) {
		size_t old = t.pool.size();
		t.pool.resize(old + 512);
		for (size_t i = old; i < t.pool.size(); i++) cudaEventCreate(&t.pool[i]);
	}
	slot = (int)t.used.size() * 2;
	t.used.push_back({kind, slot});
	cudaEventRecord(t.pool[slot], c->stream);
	return t.pool[slot];
}
void timing_end(mf_ctx* c, int slot, uint64_t rows) {
	if (slot < 0) return;
	Timing& t = c->timing;
	cudaEventRecord(t.pool[slot + 1], c->stream);
	int kind = t.used[slot / 2].first;
	t.launches[kind]++;
	t.rows[kind] += rows;
}
// Reserve an event pair for a launcher that records the events itself.
int timing_reserve(mf_ctx* c, int kind) {
	int slot;
	if (!c->timing.on) return -1;
	timing_begin(c, kind, slot);  // records the start event now; the launcher re-records both
	return slot;
}
void timing_count(mf_ctx* c, int slot, uint64_t rows) {
	if (slot < 0) return;
	Timing& t = c->timing;
	int kind = t.used[slot / 2].first;
	t.launches[kind]++;
	t.rows[kind] += rows;
}
void timing_collect(mf_ctx* c) {
	Timing& t = c->timing;
	for (auto& u : t.used) {
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, t.pool[u.second], t.pool[u.second + 1]) == cudaSuccess) t.ms[u.first] += ms;
	}
	t.used.clear();
}

mf_status check_status(mf_ctx* c) {
	CK(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(DevStatusH), cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	if (c->timing.on) timing_collect(c);
	DevStatusH s = *c->h_status;
	if (s.flags == 0) return MF_OK;
	// clear for the next call
	c->h_status->flags = 0;
	c->h_status->first_index = 0xffffffffu;
	CK(cudaMemcpyAsync(c->d_status, c->h_status, sizeof(DevStatusH), cudaMemcpyHostToDevice, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	// the root cause first: a non-finite state also breaks the grid and the neighbour search
	if (s.flags & 8u) return fail(c, MF_ERR_NONFINITE, "non-finite state at row %u", s.first_index);
	if (s.flags & 16u) return fail(c, MF_ERR_SINGULAR, "singular corrector matrix at row %u", s.first_index);
	if (s.flags & 4u) return fail(c, MF_ERR_GRID, "cell grid invalid (num_cell >= n or particle outside) near row %u", s.first_index);
	if (s.flags & 1u) return fail(c, MF_ERR_NBH_OVERFLOW, "neighbour capacity reached at row %u", s.first_index);
	if (s.flags & 2u) return fail(c, MF_ERR_NO_NEIGHBOR, "particle without neighbours at row %u", s.first_index);
	if (s.flags & 32u) return fail(c, MF_ERR_TIMEOUT, "bounded device wait gave up");
	return fail(c, MF_ERR_CUDA, "device status 0x%x", s.flags);
}

// With per-body masking: MF_ERR_BODY_FAILED while any body has failed (the others
// have stepped on), else MF_OK.
mf_status failed_status(mf_ctx* c) {
	if (!c->mask_failed || !c->ready) return MF_OK;
	const uint32_t nb = (uint32_t)c->bodies.size();
	std::vector<uint32_t> f(nb);
	CK(cudaMemcpy(f.data(), c->failed.p, (size_t)nb * 4, cudaMemcpyDeviceToHost));
	uint32_t cnt = 0, first = nb;
	for (uint32_t b = 0; b < nb; b++)
		if (f[b]) {
			cnt++;
			if (first == nb) first = b;
		}
	if (!cnt) return MF_OK;
	return fail(c, MF_ERR_BODY_FAILED, "%u of %u bodies failed and are frozen (first: body %u, flags 0x%x)", cnt, nb,
	            first, f[first]);
}

// ---------------------------------------------------------------- set-up
mf_status finalize(mf_ctx* c) {
	if (c->ready) return MF_OK;
	if (c->bodies.empty()) return fail(c, MF_ERR_STATE, "no bodies");
	const std::vector<int32_t>& acts = c->bodies[0].actions;
	for (auto& b : c->bodies)
		if (b.actions != acts) return fail(c, MF_ERR_PIPELINE, "all bodies of a context must share one action list");
	c->mixed = c->cfg.precision == MF_PREC_MIXED;
	c->strict = c->cfg.precision == MF_PREC_FP64_STRICT;
	// the weak UL form's mixed precision lives in its neighbourhood kernel alone: its
	// state and passes stay FP64
	c->uw_mixed = c->mixed && c->cfg.method == MF_METHOD_UL_WEAK;
	if (c->uw_mixed) c->mixed = false;
	mf_status st = MF_OK;
	if (c->cfg.method == MF_METHOD_UL) {
		st = validate_ul(c, acts, c->flags);
	} else if (c->cfg.method == MF_METHOD_TL) {
		st = validate_tl(c, acts, c->flags);
	} else if (c->cfg.method == MF_METHOD_COROT) {
		st = validate_corot(c, acts, c->flags);
	} else if (c->cfg.method == MF_METHOD_POTENTIAL) {
		st = validate_potential(c, acts, c->flags);
	} else if (c->cfg.method == MF_METHOD_UL_WEAK) {
		st = validate_ulweak(c, acts, c->flags);
	} else {
		st = validate_weak(c, acts, c->flags);
	}
	if (st != MF_OK) return st;
	// the reference's UL set-ups use the velocity form (tensile.cpp:44-66), applied after
	// each step; the TL set-ups the pull form (tensile.cpp:20-42), applied per stage
	for (auto& b : c->bodies)
		for (auto& bc : b.bcs) {
			const bool ul = c->cfg.method == MF_METHOD_UL || c->cfg.method == MF_METHOD_UL_WEAK;
			if (ul && bc.kind != MF_BC_VELOCITY)
				return fail(c, MF_ERR_PIPELINE, "updated-Lagrangian bodies take MF_BC_VELOCITY conditions");
			if (!ul && bc.kind != MF_BC_PULL)
				return fail(c, MF_ERR_PIPELINE, "total-Lagrangian bodies take MF_BC_PULL conditions");
		}

	uint32_t n = c->n_total;
	CK(c->body_of.alloc(n));
	std::vector<uint32_t> bof(n);
	for (size_t b = 0; b < c->bodies.size(); b++)
		for (uint32_t i = 0; i < c->bodies[b].n; i++) bof[c->bodies[b].off + i] = (uint32_t)b;
	CK(cudaMemcpy(c->body_of.p, bof.data(), n * 4, cudaMemcpyHostToDevice));
	CK(c->failed.alloc(c->bodies.size()));
	CK(cudaMemset(c->failed.p, 0, c->bodies.size() * 4));

	auto upload = [&](DevBuf<double>& d, int field) -> mf_status {
		CK(d.alloc(n));
		std::vector<double> v(n);
		for (auto& b : c->bodies) std::copy(b.in[field].begin(), b.in[field].end(), v.begin() + b.off);
		CK(cudaMemcpy(d.p, v.data(), n * 8, cudaMemcpyHostToDevice));
		return MF_OK;
	};
	// 0 x 1 y 2 X 3 Y 4 m 5 rho 6 h 7 qw 8 vx 9 vy 10 Sxx 11 Sxy 12 Syy
	if ((st = upload(c->m, 4)) || (st = upload(c->h, 6)) || (st = upload(c->qw0, 7)) || (st = upload(c->X, 2)) ||
	    (st = upload(c->Y, 3)))
		return st;
	CK(c->fcx.alloc(n)); CK(c->fcy.alloc(n));
	CK(cudaMemset(c->fcx.p, 0, n * 8)); CK(cudaMemset(c->fcy.p, 0, n * 8));
	const int fld[8] = {0, 1, 8, 9, 5, 10, 11, 12};
	for (int k = 0; k < 3; k++) {
		for (int q = 0; q < 8; q++) {
			bool fp64 = !c->mixed || q < 4;
			if (!fp64) continue;
			if (k == 0) {
				if ((st = upload(c->sd[0][q], fld[q]))) return st;
			} else {
				CK(c->sd[k][q].alloc(n));
				CK(cudaMemset(c->sd[k][q].p, 0, n * 8));
			}
		}
		if (c->mixed) {
			for (int q = 0; q < 4; q++) {
				CK(c->sf[k][q].alloc(n));
				if (k == 0) {
					std::vector<float> v(n);
					for (auto& b : c->bodies)
						for (uint32_t i = 0; i < b.n; i++)
							v[b.off + i] = (float)(b.in[fld[4 + q]][i] - (q == 0 ? b.sd.rho0 : 0.));
					CK(cudaMemcpy(c->sf[0][q].p, v.data(), n * 4, cudaMemcpyHostToDevice));
				} else {
					CK(cudaMemset(c->sf[k][q].p, 0, n * 4));
				}
			}
		}
	}
	c->h_params.clear();
	for (auto& b : c->bodies) c->h_params.push_back(make_params(b));
	CK(c->params.alloc(c->h_params.size()));
	CK(cudaMemcpy(c->params.p, c->h_params.data(), c->h_params.size() * sizeof(BodyParams), cudaMemcpyHostToDevice));

	CK(c->work.alloc(1));
	// UL grid machinery (also used for the UL neighbour dump)
	if (c->cfg.method == MF_METHOD_UL) {
		uint32_t nb = (uint32_t)c->bodies.size();
		CK(c->geom.alloc(nb));
		CK(c->bbox.alloc(6 * (size_t)nb));
		CK(c->total_cells.alloc(1));
		CK(c->keys.alloc(n)); CK(c->keys_sorted.alloc(n)); CK(c->perm_in.alloc(n)); CK(c->perm.alloc(n));
		// the mixed grid may use half-size cells: up to twice as many cells as particles
		c->cell_cap = c->mixed ? 3 * n + 7 : n + 1;
		CK(c->cell_start.alloc((size_t)c->cell_cap + 1));
		CK(c->rec_body.alloc(n));
		CK(c->rec.alloc((size_t)n * 128));
		if (c->mixed) CK(c->rec2.alloc((size_t)n * 128));
		int bits = 1;
		while (bits < 32 && (1ull << bits) < (uint64_t)c->cell_cap + 1) bits++;
		c->sort_bits = bits;
		size_t tmp = c->strict ? mf_strict::ul_sort_tmp_bytes(n, bits) : mf_fast::ul_sort_tmp_bytes(n, bits);
		CK(c->sort_tmp.alloc(tmp));
		if ((st = upload_bcs(c)) != MF_OK) return st;
	} else if (c->cfg.method == MF_METHOD_TL || c->cfg.method == MF_METHOD_COROT || c->cfg.method == MF_METHOD_POTENTIAL) {
		mf_status s2 = tl_setup(c);
		if (s2 != MF_OK) return s2;
	} else if (c->cfg.method == MF_METHOD_UL_WEAK) {
		mf_status s2 = uw_setup(c);
		if (s2 != MF_OK) return s2;
	} else {
		mf_status s2 = weak_setup(c);
		if (s2 != MF_OK) return s2;
	}
	{
		mf_status s2 = contact_setup(c);
		if (s2 != MF_OK) return s2;
	}
	c->ready = true;
	return MF_OK;
}

mf_status ul_step(mf_ctx* c) {
	for (uint32_t s = 0; s < 4; s++) {
		ULArgs a = ul_args(c, s);
		// kind 4: the whole stage (grid build when due, gather, pair); kind 0: the pair
		// kernel alone, between events the launcher records around it
		int slot_all, slot_pair;
		timing_begin(c, 4, slot_all);
		slot_pair = timing_reserve(c, 0);
		if (slot_pair >= 0) {
			a.ev_pair0 = c->timing.pool[slot_pair];
			a.ev_pair1 = c->timing.pool[slot_pair + 1];
		}
		cudaError_t e = c->strict ? mf_strict::ul_stage(a, c->mixed, c->stream) : mf_fast::ul_stage(a, c->mixed, c->stream);
		timing_count(c, slot_pair, c->n_total);
		timing_end(c, slot_all, c->n_total);
		if (e != cudaSuccess) return cuda_fail(c, e, "ul_stage");
		c->launches += (a.strict_grid || s == 0) ? 8 + 4 : (a.skip_gather ? 1 : 2);
	}
	if (c->n_bc) {  // rk4.h:105: the conditions act on the particles after the combine
		cudaError_t e = c->strict ? mf_strict::ul_bc(c->n_bc, c->bc_rows.p, c->bc_v.p, c->sd[0][2].p, c->sd[0][3].p, c->stream)
		                          : mf_fast::ul_bc(c->n_bc, c->bc_rows.p, c->bc_v.p, c->sd[0][2].p, c->sd[0][3].p, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "ul_bc");
		c->launches++;
	}
	return MF_OK;
}

// Halo tiles of the mixed TL passes.  Rows are ordered along a Z-order (Morton) curve
// of their reference positions, quantised at half the search h, and cut into tiles
// of TL_TILE consecutive positions: compact 2-D patches.  A tile's halo is the sorted
// set of every row its rows' lists name; each list entry becomes the entry's slot in
// that halo.  The lists stay in their ascending-j order, so each row sums exactly as
// before.  Tiles whose halo would not fit the shared-memory budget leave the untiled
// passes in use.
uint32_t morton_spread(uint32_t v) {
	v &= 0xffffu;
	v = (v | (v << 8)) & 0x00ff00ffu;
	v = (v | (v << 4)) & 0x0f0f0f0fu;
	v = (v | (v << 2)) & 0x33333333u;
	v = (v | (v << 1)) & 0x55555555u;
	return v;
}

// Mixed TL run walk: every row's list (ascending j, CSR `off` / c->nbr) as runs of
// consecutive rows, one word each (first row | (length - 1) << TL_RUN_SHIFT, at most
// TL_RUN_MAX_LEN rows per word), in sliced ELL; the reference positions as float-float
// pairs.  The rows' corrections (rw_G) come from the Randles-Libersky set-up.
mf_status build_tl_runs(mf_ctx* c, const std::vector<uint32_t>& off) {
	const uint32_t n = c->n_total;
	std::vector<uint32_t> nb(off[n]);
	if (off[n]) CK(cudaMemcpy(nb.data(), c->nbr.p, (size_t)off[n] * 4, cudaMemcpyDeviceToHost));
	std::vector<uint32_t> words;
	std::vector<uint32_t> roff(n + 1, 0);
	words.reserve(off[n] / 2 + n);
	for (uint32_t i = 0; i < n; i++) {
		roff[i] = (uint32_t)words.size();
		uint32_t q = off[i];
		while (q < off[i + 1]) {
			uint32_t j0 = nb[q], len = 1;
			while (q + len < off[i + 1] && len < TL_RUN_MAX_LEN && nb[q + len] == j0 + len) len++;
			words.push_back(j0 | ((len - 1) << TL_RUN_SHIFT));
			q += len;
		}
		if (words.size() - roff[i] > 0xffffu) return fail(c, MF_ERR_CAPACITY, "more than 65535 runs in one list");
	}
	roff[n] = (uint32_t)words.size();
	c->rw_words = words.size();
	const uint32_t ns = (n + 31) / 32;
	std::vector<uint32_t> sl(ns + 1, 0);
	uint64_t ent = 0;
	for (uint32_t s_ = 0; s_ < ns; s_++) {
		uint32_t w = 0;
		for (uint32_t r = 32 * s_; r < std::min(n, 32 * s_ + 32); r++) w = std::max(w, roff[r + 1] - roff[r]);
		sl[s_] = (uint32_t)ent;
		ent += 32ull * w;
	}
	if (ent > 0xffffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^32 sliced-ELL run entries");
	sl[ns] = (uint32_t)ent;
	std::vector<uint32_t> sell(std::max<uint64_t>(ent, 1), 0);
	std::vector<uint16_t> cnt(n);
	for (uint32_t i = 0; i < n; i++) {
		cnt[i] = (uint16_t)(roff[i + 1] - roff[i]);
		uint64_t base = sl[i >> 5] + (i & 31u);
		for (uint32_t k = 0; k < cnt[i]; k++) sell[base + 32ull * k] = words[roff[i] + k];
	}
	CK(c->rw_sl.alloc(ns + 1));
	CK(c->rw_cnt.alloc(n));
	CK(c->rw_runs.alloc(sell.size()));
	CK(c->rw_XF.alloc(n));
	CK(cudaMemcpy(c->rw_sl.p, sl.data(), (ns + 1) * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->rw_cnt.p, cnt.data(), (size_t)n * 2, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->rw_runs.p, sell.data(), sell.size() * 4, cudaMemcpyHostToDevice));
	// the positions the Randles-Libersky set-up used (the set-up state)
	cudaError_t e = mf_fast::tl_ref_positions(n, c->sd[0][0].p, c->sd[0][1].p, c->rw_XF.p, c->stream);
	if (e != cudaSuccess) return cuda_fail(c, e, "reference positions");
	CK(cudaStreamSynchronize(c->stream));
	c->rw_ok = true;
	return MF_OK;
}

mf_status build_tl_tiles(mf_ctx* c, const std::vector<uint32_t>& off) {
	const uint32_t n = c->n_total, T = TL_TILE;
	const uint32_t HALO_CAP = 2048;  // 128 KB of records in pass B
	c->tt_ok = false;
	if (n == 0) return MF_OK;
	std::vector<uint32_t> nbr(off[n]);
	CK(cudaMemcpy(nbr.data(), c->nbr.p, (size_t)off[n] * 4, cudaMemcpyDeviceToHost));
	std::vector<double> X(n), Y(n);
	for (auto& b : c->bodies) {
		std::copy(b.in[2].begin(), b.in[2].end(), X.begin() + b.off);
		std::copy(b.in[3].begin(), b.in[3].end(), Y.begin() + b.off);
	}
	double mnx = 1e300, mny = 1e300, mxx = -1e300, mxy = -1e300;
	for (uint32_t i = 0; i < n; i++) {
		mnx = std::min(mnx, X[i]); mxx = std::max(mxx, X[i]);
		mny = std::min(mny, Y[i]); mxy = std::max(mxy, Y[i]);
	}
	double ext = std::max(mxx - mnx, mxy - mny);
	double qz = 0.5 * c->cfg.nbh_h;
	if (!(qz > 0.) || ext / qz > 65535.) qz = ext > 0. ? ext / 65535. : 1.;
	std::vector<uint64_t> key(n);
	for (uint32_t i = 0; i < n; i++) {
		uint32_t ix = (uint32_t)std::min(65535., (X[i] - mnx) / qz), iy = (uint32_t)std::min(65535., (Y[i] - mny) / qz);
		key[i] = ((uint64_t)(morton_spread(ix) | (morton_spread(iy) << 1)) << 32) | i;
	}
	std::sort(key.begin(), key.end());
	std::vector<uint32_t> rows(n);
	for (uint32_t p = 0; p < n; p++) rows[p] = (uint32_t)key[p];
	key.clear();
	key.shrink_to_fit();
	const uint32_t nt = (n + T - 1) / T, ns = (n + 31) / 32;
	std::vector<uint32_t> tsl(ns + 1);
	uint64_t ent = 0;
	for (uint32_t s_ = 0; s_ < ns; s_++) {
		uint32_t w = 0;
		for (uint32_t p = 32 * s_; p < std::min(n, 32 * s_ + 32); p++) w = std::max(w, off[rows[p] + 1] - off[rows[p]]);
		tsl[s_] = (uint32_t)ent;
		ent += 32ull * w;
	}
	if (ent > 0xffffffffull) return MF_OK;
	tsl[ns] = (uint32_t)ent;
	std::vector<uint16_t> loc(ent, 0);
	std::vector<std::vector<uint32_t>> halos(nt);
	std::atomic<uint32_t> next{0};
	std::atomic<bool> too_big{false};
	auto work = [&]() {
		std::vector<uint32_t> js;
		for (uint32_t t; (t = next.fetch_add(1)) < nt;) {
			uint32_t p0 = t * T, p1 = std::min(n, p0 + T);
			js.clear();
			for (uint32_t p = p0; p < p1; p++) js.insert(js.end(), nbr.begin() + off[rows[p]], nbr.begin() + off[rows[p] + 1]);
			std::sort(js.begin(), js.end());
			js.erase(std::unique(js.begin(), js.end()), js.end());
			if (js.size() > HALO_CAP) {
				too_big = true;
				continue;
			}
			for (uint32_t p = p0; p < p1; p++) {
				uint32_t i = rows[p];
				uint64_t q = tsl[p >> 5] + (p & 31u);
				for (uint32_t k = off[i]; k < off[i + 1]; k++, q += 32)
					loc[q] = (uint16_t)(std::lower_bound(js.begin(), js.end(), nbr[k]) - js.begin());
			}
			halos[t] = js;
		}
	};
	unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
	std::vector<std::thread> pool;
	for (unsigned k = 1; k < nth; k++) pool.emplace_back(work);
	work();
	for (auto& th : pool) th.join();
	if (too_big) return MF_OK;
	std::vector<uint32_t> hoff(nt + 1, 0), halo;
	uint32_t hmax = 1;
	for (uint32_t t = 0; t < nt; t++) {
		hoff[t] = (uint32_t)halo.size();
		halo.insert(halo.end(), halos[t].begin(), halos[t].end());
		hmax = std::max(hmax, (uint32_t)halos[t].size());
	}
	hoff[nt] = (uint32_t)halo.size();
	CK(c->tt_rows.alloc(n)); CK(c->tt_halo_off.alloc(nt + 1)); CK(c->tt_halo.alloc(halo.size()));
	CK(c->tt_sl.alloc(ns + 1)); CK(c->tt_cnt.alloc(n)); CK(c->tt_loc.alloc(ent));
	CK(c->tt_sw.alloc(ent)); CK(c->tt_swA.alloc(ent));
	CK(cudaMemcpy(c->tt_rows.p, rows.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->tt_halo_off.p, hoff.data(), (size_t)(nt + 1) * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->tt_halo.p, halo.data(), halo.size() * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->tt_sl.p, tsl.data(), (size_t)(ns + 1) * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->tt_loc.p, loc.data(), (size_t)ent * 2, cudaMemcpyHostToDevice));
	cudaError_t e = c->strict ? mf_strict::tl_tile_sell(n, c->tt_rows.p, c->sl_off.p, c->scnt.p, c->sw32.p, c->swA32.p,
	                                                    c->tt_sl.p, c->tt_cnt.p, c->tt_sw.p, c->tt_swA.p, c->stream)
	                          : mf_fast::tl_tile_sell(n, c->tt_rows.p, c->sl_off.p, c->scnt.p, c->sw32.p, c->swA32.p,
	                                                  c->tt_sl.p, c->tt_cnt.p, c->tt_sw.p, c->tt_swA.p, c->stream);
	if (e != cudaSuccess) return cuda_fail(c, e, "tl_tile_sell");
	uint32_t emax = 32;
	for (uint32_t t = 0; t < nt; t++) {
		uint32_t s0 = t * (T / 32), s1 = std::min(s0 + T / 32, ns);
		emax = std::max(emax, tsl[s1] - tsl[s0]);
	}
	if (64ull * hmax > 200 * 1024) return MF_OK;  // the untiled passes stay in use
	e = c->strict ? mf_strict::tl_tile_attrs(hmax, emax) : mf_fast::tl_tile_attrs(hmax, emax);
	if (e != cudaSuccess) return cuda_fail(c, e, "tl_tile_attrs");
	CK(cudaStreamSynchronize(c->stream));
	c->tt_n_tiles = nt;
	c->tt_halo_max = hmax;
	c->tt_ent_max = emax;
	c->tt_ok = true;
	return MF_OK;
}

TLArgs tl_args(mf_ctx* c) {
	TLArgs a{};
	a.n_total = c->n_total;
	a.n_bodies = (uint32_t)c->bodies.size();
	a.flags = c->flags;
	a.params = c->params.p;
	a.body_of = c->body_of.p;
	a.X = c->X.p; a.Y = c->Y.p; a.m = c->m.p; a.h = c->h.p; a.qw0 = c->qw0.p; a.fcx = c->fcx.p; a.fcy = c->fcy.p;
	a.qw32 = c->qw32.p; a.m32 = c->m32.p; a.h32 = c->h32.p;
	StateSoA* s[4] = {&a.base, &a.acc, &a.st, &a.nxt};
	for (int k = 0; k < 4; k++) {
		double** d[8] = {&s[k]->x, &s[k]->y, &s[k]->vx, &s[k]->vy, &s[k]->rho, &s[k]->Sxx, &s[k]->Sxy, &s[k]->Syy};
		for (int q = 0; q < 8; q++) *d[q] = c->sd[k][q].p;
		s[k]->rho_f = c->sf[k][0].p; s[k]->Sxx_f = c->sf[k][1].p; s[k]->Sxy_f = c->sf[k][2].p; s[k]->Syy_f = c->sf[k][3].p;
	}
	a.sl_off = c->sl_off.p;
	a.cnt = c->scnt.p;
	a.snbr = c->snbr.p;
	a.sw = c->mixed ? (const void*)c->sw32.p : (const void*)c->sw64.p;
	a.swA = c->swA32.p;
	a.P = c->P64.p;
	a.dA = c->dA64.p;
	a.c = c->c64.p;
	a.sW = c->sW64.p;
	a.R = c->R64.p;
	a.av = c->av64.p;
	a.cm_sw = c->cm_sw.p; a.cm_swA = c->cm_swA.p; a.cm_sX = c->cm_sX.p; a.cm_sW = c->cm_sW.p; a.cm_swji = c->cm_swji.p;
	a.cm_U = c->cm_U.p; a.cm_X = c->cm_X.p; a.cm_V = c->cm_V.p; a.cm_P = c->cm_P.p; a.cm_R = c->cm_R.p;
	a.cm_H = c->cm_H.p;
	a.recA = c->recA.p;
	a.recB = c->recB.p;
	a.dA32 = c->dA32.p;
	a.bc_rows = c->bc_rows.p;
	a.bc_v = c->bc_v.p;
	a.n_bc = c->n_bc;
	a.status = c->d_status;
	a.block = c->tune.tl_block;
	if (c->mixed && c->rw_ok && c->tune.tl_runs) {
		a.r_sl = c->rw_sl.p;
		a.r_cnt = c->rw_cnt.p;
		a.runs = c->rw_runs.p;
		a.XF = c->rw_XF.p;
		a.G = c->rw_G.p;
		a.unroll = c->tune.tl_unroll;
	}
	if (c->mixed && c->tt_ok && c->tune.tl_tiled) {
		a.t_rows = c->tt_rows.p;
		a.t_halo_off = c->tt_halo_off.p;
		a.t_halo = c->tt_halo.p;
		a.t_sl = c->tt_sl.p;
		a.t_cnt = c->tt_cnt.p;
		a.t_loc = c->tt_loc.p;
		a.t_sw = c->tt_sw.p;
		a.t_swA = c->tt_swA.p;
		a.n_tiles = c->tt_n_tiles;
		a.halo_max = c->tt_halo_max;
		a.t_ent_max = c->tt_ent_max;
	}
	return a;
}

cudaError_t tl_launch(mf_ctx* c, const TLArgs& a, int part) {
	return c->strict ? mf_strict::tl_stage(a, c->mixed, part, c->stream) : mf_fast::tl_stage(a, c->mixed, part, c->stream);
}

mf_status contact_run(mf_ctx* c, cudaStream_t s);

// One RK4 step of every TL body: per stage the BCs, (pack), pass A, pass B; the
// stage state ping-pongs between sets 2 and 3 so that pass B never overwrites data
// its neighbours still read.  fork_contact: the pending contact query of the particles'
// positions (set 0, written only by stage 3) runs on the side stream beside stage 0's
// pass A, and pass B (the first reader of the forces) waits for it.
mf_status tl_step_all(mf_ctx* c, bool fork_contact = false) {
	TLArgs a = tl_args(c);
	StateSoA S0 = a.st, S1 = a.nxt;
	// mixed form: pass B writes the next stage's records (no pack kernel), except with
	// boundary conditions, which change the stage state after pass B
	const bool corot = c->cfg.method == MF_METHOD_COROT, potential = c->cfg.method == MF_METHOD_POTENTIAL;
	const bool fused = c->mixed && c->n_bc == 0 && !corot && !potential;
	void* rb[2] = {c->recB.p, c->recB2.p};
	for (uint32_t st = 0; st < 4; st++) {
		a.stage = st;
		a.st = (st % 2 == 0) ? S0 : S1;
		a.nxt = (st % 2 == 0) ? S1 : S0;
		a.recB = fused ? rb[st & 1] : rb[0];
		a.recB_out = rb[(st + 1) & 1];
		a.write_recs = fused ? 1u : 0u;
		const bool pack = c->mixed && !corot && !potential && (!fused || (st == 0 && !c->tl_recs_valid));
		cudaError_t e;
		if ((e = tl_launch(c, a, 0)) != cudaSuccess) return cuda_fail(c, e, "tl bc");
		if (pack && (e = tl_launch(c, a, 1)) != cudaSuccess) return cuda_fail(c, e, "tl pack");
		int slot;
		if (corot || potential) {
			auto cr = [&](int part) {
				return c->strict ? mf_strict::cr_stage(a, part, c->stream) : mf_fast::cr_stage(a, part, c->stream);
			};
			const int base = c->mixed ? 10 : 0;  // the mixed form's records, then its passes
			if (c->mixed && (e = cr(10)) != cudaSuccess) return cuda_fail(c, e, "records");
			if (corot && (e = cr(base + (c->mixed ? 1 : 0))) != cudaSuccess) return cuda_fail(c, e, "corotational rotation");
			timing_begin(c, 1, slot);
			if ((e = cr(base + (c->mixed ? 2 : 1))) != cudaSuccess) return cuda_fail(c, e, "pass A");
			timing_end(c, slot, c->n_total);
			timing_begin(c, 2, slot);
			if ((e = cr(base + (c->mixed ? 3 : 2))) != cudaSuccess) return cuda_fail(c, e, "pass B");
			timing_end(c, slot, c->n_total);
			c->launches += (corot ? 3 : 2) + (c->mixed ? 1 : 0) + (c->n_bc ? 1 : 0);
			continue;
		}
		const bool fork = fork_contact && st == 0;
		if (fork) {
			CK(cudaEventRecord(c->ev_fork, c->stream));
			CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
			mf_status cs = contact_run(c, c->side);
			if (cs != MF_OK) return cs;
			CK(cudaEventRecord(c->ev_join, c->side));
		}
		timing_begin(c, 1, slot);
		if ((e = tl_launch(c, a, 2)) != cudaSuccess) return cuda_fail(c, e, "tl pass A");
		timing_end(c, slot, c->n_total);
		if (fork) CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
		timing_begin(c, 2, slot);
		if ((e = tl_launch(c, a, 3)) != cudaSuccess) return cuda_fail(c, e, "tl pass B");
		timing_end(c, slot, c->n_total);
		c->launches += 2 + (c->n_bc ? 1 : 0) + (pack ? 1 : 0);
	}
	if (fused) c->tl_recs_valid = true;
	cudaError_t e;
	if ((e = tl_launch(c, a, 4)) != cudaSuccess) return cuda_fail(c, e, "tl bc");
	if ((e = tl_launch(c, a, 5)) != cudaSuccess) return cuda_fail(c, e, "tl clock");
	c->launches += 1 + (c->n_bc ? 1 : 0);
	return MF_OK;
}

// Mixed TL: pack the stage-0 records now (outside a graph capture), so that the
// captured step needs no pack kernel.
mf_status tl_prepack(mf_ctx* c) {
	if (c->cfg.method != MF_METHOD_TL || !c->mixed || c->n_bc || c->tl_recs_valid) return MF_OK;
	TLArgs a = tl_args(c);
	a.stage = 0;
	a.recB = c->recB.p;
	cudaError_t e = tl_launch(c, a, 1);
	if (e != cudaSuccess) return cuda_fail(c, e, "tl pack");
	c->launches++;
	c->tl_recs_valid = true;
	return MF_OK;
}

// Corotational pipeline (rings.cpp:325-331, tensile.cpp:202-208, rotation.cpp:132-137):
// the rotation, displacement, Cauchy-Green stress, nominal stress and stress actions
// in this order, then optionally the artificial viscosity and advection.
mf_status validate_corot(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_COROTATIONAL_ANISOTROPY_TENSOR, MF_DERIVE_DISPLACEMENT_COROTATIONAL,
	                            MF_MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN, MF_CONTMECH_CAUCHY_TO_NOMINAL,
	                            MF_DERIVE_STRESS_COROTATIONAL, MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
	                            MF_CONTMECH_ADVECTION};
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not part of the corotational pipeline or out of its order", a);
		flags |= abit(a);
		pos++;
	}
	for (int k = 0; k < 5; k++)
		if (!(flags & abit(order[k])))
			return fail(c, MF_ERR_PIPELINE, "the corotational pipeline needs action %d", order[k]);
	return MF_OK;
}

// Elastic-potential pipeline (rings.cpp:512-516, tensile.cpp:354-358,
// rotation.cpp:266-269): displacement, Green-St Venant stress, the potential forces,
// then optionally the artificial viscosity and advection.
mf_status validate_potential(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_DERIVE_DISPLACEMENT, MF_MATERIAL_COMPUTE_STRESS_GREEN_STVENANT,
	                            MF_POTENTIAL_COMP_ELASTIC_POTENTIAL, MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
	                            MF_CONTMECH_ADVECTION};
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not part of the elastic-potential pipeline or out of its order", a);
		flags |= a == MF_POTENTIAL_COMP_ELASTIC_POTENTIAL ? FLAG_POTENTIAL : abit(a);
		pos++;
	}
	if (!(flags & FLAG_POTENTIAL))
		return fail(c, MF_ERR_PIPELINE, "the elastic-potential pipeline needs potential_comp_elastic_potential");
	return MF_OK;
}

// TL pipeline: a subsequence of the union of the reference's two TL lists
// (rings.cpp:419-425 and tensile.cpp:276-286) in this order.
mf_status validate_tl(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_DERIVE_DISPLACEMENT, MF_DERIVE_VELOCITY_TL, MF_CONTMECH_VELOCITY_GRADIENT_TL,
	                            MF_CONTMECH_CONTINUITY, MF_MATERIAL_EOS, MF_MATERIAL_STRESS_RATE_JAUMANN,
	                            MF_MATERIAL_COMPUTE_STRESS_GREEN_STVENANT, MF_CONTMECH_CAUCHY_TO_NOMINAL,
	                            MF_DERIVE_STRESS_TL, MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY, MF_CONTMECH_MOMENTUM_TL,
	                            MF_CONTMECH_ADVECTION};
	if (c->cfg.method != MF_METHOD_TL) return fail(c, MF_ERR_PIPELINE, "method %d is not available", c->cfg.method);
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not part of the fused TL pipeline or out of its order", a);
		flags |= abit(a);
		pos++;
	}
	if ((flags & abit(MF_CONTMECH_MOMENTUM_TL)) && !(flags & abit(MF_DERIVE_STRESS_TL)))
		return fail(c, MF_ERR_PIPELINE, "contmech_momentum_tl needs derive_stress_tl before it");
	if ((flags & abit(MF_CONTMECH_VELOCITY_GRADIENT_TL)) && !(flags & abit(MF_DERIVE_VELOCITY_TL)))
		return fail(c, MF_ERR_PIPELINE, "contmech_velocity_gradient_tl needs derive_velocity_tl before it");
	if ((flags & (abit(MF_CONTMECH_CONTINUITY) | abit(MF_MATERIAL_STRESS_RATE_JAUMANN))) &&
	    !(flags & abit(MF_CONTMECH_VELOCITY_GRADIENT_TL)))
		return fail(c, MF_ERR_PIPELINE, "continuity / Jaumann rate need contmech_velocity_gradient_tl before them");
	return MF_OK;
}

// TL set-up: neighbour lists (find_neighbors), Randles-Libersky gradients, stage
// buffers.  Runs once, before the first step.
mf_status tl_setup(mf_ctx* c) {
	uint32_t n = c->n_total;
	uint32_t nb = (uint32_t)c->bodies.size();
	double h = c->cfg.nbh_h, eps = c->cfg.nbh_eps;
	if (!(h > 0.)) return fail(c, MF_ERR_ARG, "TL needs config.nbh_h > 0 (the h of the set-up neighbour search)");
	double reach = sqrt(h * h * 2 * 2 + eps) * (1. + 1e-9);
	std::vector<Geom> g(nb);
	uint32_t cells = 0;
	for (uint32_t b = 0; b < nb; b++) {
		const HostBody& B = c->bodies[b];
		double mnx = 1e300, mny = 1e300, mxx = -1e300, mxy = -1e300;
		for (uint32_t i = 0; i < B.n; i++) {
			mnx = std::min(mnx, B.in[0][i]); mxx = std::max(mxx, B.in[0][i]);
			mny = std::min(mny, B.in[1][i]); mxy = std::max(mxy, B.in[1][i]);
		}
		double fnx = floor((mxx - mnx) / reach) + 1, fny = floor((mxy - mny) / reach) + 1;
		if (fnx * fny > 1.5e9) return fail(c, MF_ERR_CAPACITY, "set-up grid too large");
		g[b].bbmin_x = mnx; g[b].bbmin_y = mny; g[b].dx = reach;
		g[b].nx = (uint32_t)fnx; g[b].ny = (uint32_t)fny;
		g[b].num_cell = g[b].nx * g[b].ny;
		g[b].cell_off = cells;
		if ((uint64_t)cells + g[b].num_cell > 0xfffffff0ull) return fail(c, MF_ERR_CAPACITY, "set-up grid too large");
		cells += g[b].num_cell;
	}
	DevBuf<Geom> dgeom;
	DevBuf<uint32_t> keys, keys_sorted, vals, perm, cstart, count;
	DevBuf<unsigned char> tmp;
	CK(dgeom.alloc(nb));
	CK(cudaMemcpy(dgeom.p, g.data(), nb * sizeof(Geom), cudaMemcpyHostToDevice));
	CK(keys.alloc(n)); CK(keys_sorted.alloc(n)); CK(vals.alloc(n)); CK(perm.alloc(n));
	CK(cstart.alloc((size_t)cells + 2)); CK(count.alloc(n));
	int bits = 1;
	while (bits < 32 && (1ull << bits) < (uint64_t)cells + 2) bits++;
	size_t tb = c->strict ? mf_strict::tl_sort_tmp_bytes(n, bits) : mf_fast::tl_sort_tmp_bytes(n, bits);
	CK(tmp.alloc(tb));
	TLSearchArgs sa{};
	sa.n_from = n; sa.n_to = n;
	sa.fx = c->sd[0][0].p; sa.fy = c->sd[0][1].p; sa.tx = c->sd[0][0].p; sa.ty = c->sd[0][1].p;
	sa.from_body = c->body_of.p; sa.to_body = c->body_of.p;
	sa.geom = dgeom.p; sa.total_cells = cells;
	sa.h = h; sa.eps = eps; sa.max_nbh = c->cfg.max_nbh;
	sa.keys = keys.p; sa.keys_sorted = keys_sorted.p; sa.vals = vals.p; sa.perm = perm.p; sa.cell_start = cstart.p;
	sa.sort_tmp = tmp.p; sa.sort_tmp_bytes = tb; sa.sort_bits = bits;
	sa.count = count.p; sa.status = c->d_status;
	auto search = [&](int pass) { return c->strict ? mf_strict::tl_search(sa, pass, c->stream) : mf_fast::tl_search(sa, pass, c->stream); };
	CK(search(0));
	mf_status st = check_status(c);
	if (st != MF_OK) return st;
	std::vector<uint32_t> hc(n), off(n + 1, 0);
	CK(cudaMemcpy(hc.data(), count.p, n * 4, cudaMemcpyDeviceToHost));
	uint64_t tot = 0;
	for (uint32_t i = 0; i < n; i++) { off[i] = (uint32_t)tot; tot += hc[i]; }
	if (tot > 0xffffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^32 neighbour pairs");
	off[n] = (uint32_t)tot;
	CK(c->nbr_off.alloc(n + 1));
	CK(cudaMemcpy(c->nbr_off.p, off.data(), (n + 1) * 4, cudaMemcpyHostToDevice));
	CK(c->nbr.alloc(tot));
	sa.off = c->nbr_off.p;
	sa.nbr = c->nbr.p;
	CK(search(1));
	dgeom.free(); keys.free(); keys_sorted.free(); vals.free(); perm.free(); cstart.free(); count.free(); tmp.free();
	// Randles-Libersky corrected gradients, FP64
	CK(c->wx64.alloc(tot)); CK(c->wy64.alloc(tot));
	DevBuf<double> rho_tmp;  // the mixed form keeps no FP64 density; the set-up needs one
	if (c->mixed) {
		CK(rho_tmp.alloc(n));
		std::vector<double> v(n);
		for (auto& b : c->bodies) std::copy(b.in[5].begin(), b.in[5].end(), v.begin() + b.off);
		CK(cudaMemcpy(rho_tmp.p, v.data(), (size_t)n * 8, cudaMemcpyHostToDevice));
	}
	const double* rho64 = c->mixed ? rho_tmp.p : c->sd[0][4].p;
	const float* rho32 = nullptr;
	const bool corot = c->cfg.method == MF_METHOD_COROT, potential = c->cfg.method == MF_METHOD_POTENTIAL;
	// mixed TL: the run-walk passes (their run words address rows below 2^27)
	const bool run_walk = c->mixed && !corot && !potential && n < TL_RUN_MAX_ROWS;
	c->rw_ok = false;
	DevBuf<double> w64;  // corotational: the kernel values of the pairs (precomp_sph)
	cudaError_t e;
	if (corot) {
		CK(w64.alloc(tot));
		e = c->strict ? mf_strict::cr_sph(n, c->nbr_off.p, c->nbr.p, c->sd[0][0].p, c->sd[0][1].p, c->h.p, w64.p,
		                                  c->wx64.p, c->wy64.p, c->stream)
		              : mf_fast::cr_sph(n, c->nbr_off.p, c->nbr.p, c->sd[0][0].p, c->sd[0][1].p, c->h.p, w64.p,
		                                c->wx64.p, c->wy64.p, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "precomp_sph");
	} else {
		if (run_walk) CK(c->rw_G.alloc(n));
		e = c->strict ? mf_strict::tl_rl(n, c->nbr_off.p, c->nbr.p, c->sd[0][0].p, c->sd[0][1].p, c->m.p, rho64, rho32,
		                                 c->h.p, c->wx64.p, c->wy64.p, nullptr, c->d_status, c->stream)
		              : mf_fast::tl_rl(n, c->nbr_off.p, c->nbr.p, c->sd[0][0].p, c->sd[0][1].p, c->m.p, rho64, rho32,
		                               c->h.p, c->wx64.p, c->wy64.p, run_walk ? (void*)c->rw_G.p : nullptr, c->d_status,
		                               c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "tl_rl");
	}
	st = check_status(c);
	if (st != MF_OK) return st;
	// sliced ELL: slices of 32 rows, each padded to its longest list
	uint32_t ns = (n + 31) / 32;
	std::vector<uint32_t> sl(ns + 1, 0);
	uint64_t ent = 0;
	for (uint32_t s_ = 0; s_ < ns; s_++) {
		uint32_t w = 0;
		for (uint32_t r = 32 * s_; r < std::min(n, 32 * s_ + 32); r++) w = std::max(w, hc[r]);
		sl[s_] = (uint32_t)ent;
		ent += 32ull * w;
	}
	if (ent > 0xffffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^32 sliced-ELL entries");
	sl[ns] = (uint32_t)ent;
	CK(c->sl_off.alloc(ns + 1));
	CK(cudaMemcpy(c->sl_off.p, sl.data(), (ns + 1) * 4, cudaMemcpyHostToDevice));
	CK(c->scnt.alloc(n));
	CK(c->snbr.alloc(ent));
	const bool fam = corot || potential;       // their mixed lists come from the FP64 ones
	const bool tl_mixed_lists = c->mixed && !fam;
	if (tl_mixed_lists) {
		CK(c->sw32.alloc(ent));
		CK(c->swA32.alloc(ent));
	} else {
		CK(c->sw64.alloc(ent));
	}
	e = c->strict ? mf_strict::tl_to_sell(n, c->nbr_off.p, c->nbr.p, c->wx64.p, c->wy64.p, c->sl_off.p, c->scnt.p,
	                                      c->snbr.p, c->sw64.p, nullptr, nullptr, c->qw0.p, c->m.p, c->stream)
	              : mf_fast::tl_to_sell(n, c->nbr_off.p, c->nbr.p, c->wx64.p, c->wy64.p, c->sl_off.p, c->scnt.p,
	                                    c->snbr.p, tl_mixed_lists ? nullptr : (void*)c->sw64.p,
	                                    tl_mixed_lists ? (void*)c->sw32.p : nullptr,
	                                    tl_mixed_lists ? (void*)c->swA32.p : nullptr, c->qw0.p, c->m.p, c->stream);
	if (e != cudaSuccess) return cuda_fail(c, e, "tl_to_sell");
	if (corot) {
		CK(c->sW64.alloc(ent));
		CK(c->R64.alloc(4 * (size_t)n));
		CK(c->av64.alloc(8 * (size_t)n));
		e = c->strict ? mf_strict::cr_sell_w(n, c->nbr_off.p, c->sl_off.p, w64.p, c->sW64.p, c->stream)
		              : mf_fast::cr_sell_w(n, c->nbr_off.p, c->sl_off.p, w64.p, c->sW64.p, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "corotational weights");
	}
	if (potential) {  // precomp_randles_libersky_symmetric: the reverse pairs' gradients
		CK(c->sW64.alloc(2 * ent));
		CK(c->av64.alloc(8 * (size_t)n));
		e = c->strict ? mf_strict::cr_sell_wji(n, c->nbr_off.p, c->nbr.p, c->wx64.p, c->wy64.p, c->sl_off.p, c->sW64.p,
		                                       c->stream)
		              : mf_fast::cr_sell_wji(n, c->nbr_off.p, c->nbr.p, c->wx64.p, c->wy64.p, c->sl_off.p, c->sW64.p,
		                                     c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "reverse-pair weights");
	}
	if (fam && c->mixed) {  // FP32 per-pair arrays and per-row records of the mixed passes
		CK(c->cm_sw.alloc(ent)); CK(c->cm_swA.alloc(ent));
		if (corot) { CK(c->cm_sX.alloc(ent)); CK(c->cm_sW.alloc(ent)); CK(c->cm_R.alloc(n)); }
		else CK(c->cm_swji.alloc(ent));
		CK(c->cm_U.alloc(n)); CK(c->cm_X.alloc(n)); CK(c->cm_V.alloc(n)); CK(c->cm_P.alloc(n)); CK(c->cm_H.alloc(n));
		e = mf_fast::cr_mixed_lists(n, c->sl_off.p, c->scnt.p, c->snbr.p, c->sw64.p, c->sW64.p, potential ? 1 : 0,
		                            c->X.p, c->Y.p, c->m.p, c->qw0.p, c->cm_sw.p, c->cm_swA.p, c->cm_sX.p, c->cm_sW.p,
		                            c->cm_swji.p, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "mixed lists");
	}
	CK(cudaStreamSynchronize(c->stream));
	if (fam && c->mixed) { c->sw64.free(); c->sW64.free(); }
	c->wx64.free();
	c->wy64.free();
	if (c->mixed && !fam && c->tune.tl_tiled && (st = build_tl_tiles(c, off)) != MF_OK) return st;
	if (run_walk && (st = build_tl_runs(c, off)) != MF_OK) return st;
	if (c->mixed) {
		CK(c->recA.alloc(n)); CK(c->recB.alloc(4 * (size_t)n)); CK(c->recB2.alloc(4 * (size_t)n)); CK(c->dA32.alloc(n));
		c->tl_recs_valid = false;
		auto f32 = [&](DevBuf<float>& d, int field) -> mf_status {
			CK(d.alloc(n));
			std::vector<float> v(n);
			for (auto& b : c->bodies)
				for (uint32_t i = 0; i < b.n; i++) v[b.off + i] = (float)b.in[field][i];
			CK(cudaMemcpy(d.p, v.data(), n * 4, cudaMemcpyHostToDevice));
			return MF_OK;
		};
		if ((st = f32(c->qw32, 7)) || (st = f32(c->m32, 4)) || (st = f32(c->h32, 6))) return st;
	} else {
		CK(c->P64.alloc(4 * (size_t)n)); CK(c->dA64.alloc(4 * (size_t)n)); CK(c->c64.alloc(n));
	}
	// the second stage buffer set; stage 0 starts from a copy of the particles
	for (int q = 0; q < 8; q++) {
		if (c->mixed && q >= 4) continue;
		CK(c->sd[3][q].alloc(n));
		CK(cudaMemcpy(c->sd[2][q].p, c->sd[0][q].p, n * 8, cudaMemcpyDeviceToDevice));
	}
	if (c->mixed)
		for (int q = 0; q < 4; q++) {
			CK(c->sf[3][q].alloc(n));
			CK(cudaMemcpy(c->sf[2][q].p, c->sf[0][q].p, n * 4, cudaMemcpyDeviceToDevice));
		}
	return upload_bcs(c);
}

// The rows and speeds of every body's boundary conditions, concatenated.
mf_status upload_bcs(mf_ctx* c) {
	std::vector<uint32_t> rows;
	std::vector<double> vs;
	for (auto& b : c->bodies)
		for (auto& bc : b.bcs)
			for (uint32_t i : bc.idx) { rows.push_back(b.off + i); vs.push_back(bc.v); }
	c->n_bc = (uint32_t)rows.size();
	CK(c->bc_rows.alloc(rows.size())); CK(c->bc_v.alloc(vs.size()));
	if (!rows.empty()) {
		CK(cudaMemcpy(c->bc_rows.p, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->bc_v.p, vs.data(), vs.size() * 8, cudaMemcpyHostToDevice));
	}
	return MF_OK;
}

// Neighbour lists (find_neighbors semantics: every "from" point within
// sqrt(4h^2 + eps) of a "to" point, ascending) as CSR, over a per-body cell grid of the
// particle bounding boxes whose cell is the search radius.  `to` points must lie in
// (or near) their body's particle box.
mf_status build_lists(mf_ctx* c, const double* fx, const double* fy, const uint32_t* from_body, uint32_t n_from,
                      const double* tx, const double* ty, const uint32_t* to_body, uint32_t n_to, uint32_t cap,
                      DevBuf<uint32_t>& off_out, DevBuf<uint32_t>& nbr_out, std::vector<uint32_t>& counts,
                      bool manhattan) {
	uint32_t nb = (uint32_t)c->bodies.size();
	double h = c->cfg.nbh_h, eps = c->cfg.nbh_eps;
	// the cell covers the predicate's reach: the radius, or the Manhattan half-width
	double reach = (manhattan ? 2. * h + 1e-6 : sqrt(h * h * 2 * 2 + eps)) * (1. + 1e-9);
	std::vector<Geom> g(nb);
	uint32_t cells = 0;
	for (uint32_t b = 0; b < nb; b++) {
		const HostBody& B = c->bodies[b];
		double mnx = 1e300, mny = 1e300, mxx = -1e300, mxy = -1e300;
		for (uint32_t i = 0; i < B.n; i++) {
			mnx = std::min(mnx, B.in[0][i]); mxx = std::max(mxx, B.in[0][i]);
			mny = std::min(mny, B.in[1][i]); mxy = std::max(mxy, B.in[1][i]);
		}
		double fnx = floor((mxx - mnx) / reach) + 1, fny = floor((mxy - mny) / reach) + 1;
		if (fnx * fny > 1.5e9) return fail(c, MF_ERR_CAPACITY, "set-up grid too large");
		g[b].bbmin_x = mnx; g[b].bbmin_y = mny; g[b].dx = reach;
		g[b].nx = (uint32_t)fnx; g[b].ny = (uint32_t)fny;
		g[b].num_cell = g[b].nx * g[b].ny;
		g[b].cell_off = cells;
		if ((uint64_t)cells + g[b].num_cell > 0xfffffff0ull) return fail(c, MF_ERR_CAPACITY, "set-up grid too large");
		cells += g[b].num_cell;
	}
	DevBuf<Geom> dgeom;
	DevBuf<uint32_t> keys, keys_sorted, vals, perm, cstart, count;
	DevBuf<unsigned char> tmp;
	CK(dgeom.alloc(nb));
	CK(cudaMemcpy(dgeom.p, g.data(), nb * sizeof(Geom), cudaMemcpyHostToDevice));
	CK(keys.alloc(n_from)); CK(keys_sorted.alloc(n_from)); CK(vals.alloc(n_from)); CK(perm.alloc(n_from));
	CK(cstart.alloc((size_t)cells + 2)); CK(count.alloc(n_to));
	int bits = 1;
	while (bits < 32 && (1ull << bits) < (uint64_t)cells + 2) bits++;
	size_t tb = c->strict ? mf_strict::tl_sort_tmp_bytes(n_from, bits) : mf_fast::tl_sort_tmp_bytes(n_from, bits);
	CK(tmp.alloc(tb));
	TLSearchArgs sa{};
	sa.n_from = n_from; sa.n_to = n_to;
	sa.fx = fx; sa.fy = fy; sa.tx = tx; sa.ty = ty;
	sa.from_body = from_body; sa.to_body = to_body;
	sa.geom = dgeom.p; sa.total_cells = cells;
	sa.h = h; sa.eps = eps; sa.max_nbh = cap;
	sa.keys = keys.p; sa.keys_sorted = keys_sorted.p; sa.vals = vals.p; sa.perm = perm.p; sa.cell_start = cstart.p;
	sa.sort_tmp = tmp.p; sa.sort_tmp_bytes = tb; sa.sort_bits = bits;
	sa.count = count.p; sa.status = c->d_status;
	sa.manhattan = manhattan ? 1u : 0u;
	auto search = [&](int pass) { return c->strict ? mf_strict::tl_search(sa, pass, c->stream) : mf_fast::tl_search(sa, pass, c->stream); };
	CK(search(0));
	mf_status st = check_status(c);
	if (st != MF_OK) return st;
	counts.assign(n_to, 0);
	CK(cudaMemcpy(counts.data(), count.p, (size_t)n_to * 4, cudaMemcpyDeviceToHost));
	std::vector<uint32_t> off(n_to + 1, 0);
	uint64_t tot = 0;
	for (uint32_t i = 0; i < n_to; i++) { off[i] = (uint32_t)tot; tot += counts[i]; }
	if (tot > 0xffffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^32 neighbour pairs");
	off[n_to] = (uint32_t)tot;
	CK(off_out.alloc((size_t)n_to + 1));
	CK(cudaMemcpy(off_out.p, off.data(), ((size_t)n_to + 1) * 4, cudaMemcpyHostToDevice));
	CK(nbr_out.alloc(tot));
	sa.off = off_out.p;
	sa.nbr = nbr_out.p;
	CK(search(1));
	CK(cudaStreamSynchronize(c->stream));
	dgeom.free(); keys.free(); keys_sorted.free(); vals.free(); perm.free(); cstart.free(); count.free(); tmp.free();
	return MF_OK;
}

// Sliced-ELL offsets from per-row counts (slices of 32 rows, padded to the longest).
mf_status sell_offsets(mf_ctx* c, const std::vector<uint32_t>& counts, DevBuf<uint32_t>& sl, uint64_t& ent) {
	uint32_t n = (uint32_t)counts.size();
	uint32_t ns = (n + 31) / 32;
	std::vector<uint32_t> h(ns + 1, 0);
	ent = 0;
	for (uint32_t s_ = 0; s_ < ns; s_++) {
		uint32_t w = 0;
		for (uint32_t r = 32 * s_; r < std::min(n, 32 * s_ + 32); r++) w = std::max(w, counts[r]);
		h[s_] = (uint32_t)ent;
		ent += 32ull * w;
	}
	if (ent > 0xffffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^32 sliced-ELL entries");
	h[ns] = (uint32_t)ent;
	CK(sl.alloc(ns + 1));
	CK(cudaMemcpy(sl.p, h.data(), (ns + 1) * 4, cudaMemcpyHostToDevice));
	return MF_OK;
}

// Weak-form pipeline: a subsequence of the tensile_tl_weak list (tensile.cpp:814-823).
mf_status validate_weak(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_DERIVE_DISPLACEMENT_WEAK, MF_DERIVE_VELOCITY_TL_WEAK, MF_CONTMECH_VELOCITY_GRADIENT_TL_GP,
	                            MF_CONTMECH_CONTINUITY_GP, MF_MATERIAL_EOS_GP, MF_MATERIAL_STRESS_RATE_JAUMANN_GP,
	                            MF_CONTMECH_CAUCHY_TO_NOMINAL_GP, MF_DERIVE_STRESS_WEAK_TL, MF_CONTMECH_MOMENTUM_TL_WEAK,
	                            MF_CONTMECH_ADVECTION};
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not part of the fused weak-form pipeline or out of its order", a);
		flags |= abit(a);
		pos++;
	}
	if ((flags & abit(MF_CONTMECH_MOMENTUM_TL_WEAK)) && !(flags & abit(MF_DERIVE_STRESS_WEAK_TL)))
		return fail(c, MF_ERR_PIPELINE, "contmech_momentum_tl_weak needs derive_stress_weak_tl before it");
	if ((flags & abit(MF_CONTMECH_VELOCITY_GRADIENT_TL_GP)) && !(flags & abit(MF_DERIVE_VELOCITY_TL_WEAK)))
		return fail(c, MF_ERR_PIPELINE, "the Gauss-point velocity gradient needs derive_velocity_tl_weak before it");
	for (auto& b : c->bodies) {
		if ((b.ex == 0 || b.ey == 0) && b.quads.empty())
			return fail(c, MF_ERR_STATE, "a TL_WEAK body needs mf_set_gauss_mesh or mf_set_elements");
		if (b.shape != c->bodies[0].shape)
			return fail(c, MF_ERR_PIPELINE, "all TL_WEAK bodies take the same shape-function kind");
		const uint64_t ne = b.quads.empty() ? (uint64_t)b.ex * b.ey : b.quads.size() / 4;
		const uint64_t ngp = ne * (b.quads.empty() ? 4u : b.order * b.order);
		if (!b.gpt[0].empty() && (b.quads.empty() || b.gpt[0].size() != ngp))
			return fail(c, MF_ERR_ARG, "mf_set_gauss_points gave %zu points; the element map has %llu", b.gpt[0].size(),
			            (unsigned long long)ngp);
		if (b.gpt[0].empty() && (!(b.gp_h > 0.) || !(b.gp_rho > 0.)))
			return fail(c, MF_ERR_ARG, "Gauss-point h and rho must be positive (or given by mf_set_gauss_points)");
	}
	return MF_OK;
}

// Element map of a weak TL body: the explicit one, or element_map_rectangle(ex, ey)
// (element.cpp:23-39: row-major elements, nodes ll lr tr tl), in global particle indices.
static void body_quads(const HostBody& B, std::vector<uint32_t>& q) {
	if (!B.quads.empty()) {
		for (uint32_t k : B.quads) q.push_back(B.off + k);
		return;
	}
	const uint32_t nx = B.ex + 1;
	for (uint32_t i = 0; i < B.ey; i++)
		for (uint32_t j = 0; j < B.ex; j++) {
			uint32_t ll = B.off + i * nx + j;
			q.push_back(ll); q.push_back(ll + 1); q.push_back(ll + nx + 1); q.push_back(ll + nx);
		}
}

// Weak-form set-up (tensile.cpp:776-807, rings.cpp:742-790, rotation.cpp:425-440): Gauss
// points on the element maps, the lists of Gauss points and particles (RKPM on
// neighbourhoods, or the elements' own functions), the transposed Gauss-point lists,
// sliced ELL.
mf_status weak_setup(mf_ctx* c) {
	uint32_t n = c->n_total;
	uint32_t nb = (uint32_t)c->bodies.size();
	const bool fem = c->bodies[0].shape == MF_SHAPE_ELEMENT;
	if (!fem && !(c->cfg.nbh_h > 0.)) return fail(c, MF_ERR_ARG, "TL_WEAK with RKPM needs config.nbh_h > 0");
	std::vector<uint32_t> quads, gpb, b_order(nb), b_eoff(nb + 1), b_goff(nb + 1);
	std::vector<double> gh, grho;
	uint64_t ng64 = 0;
	for (uint32_t b = 0; b < nb; b++) {
		const HostBody& B = c->bodies[b];
		b_eoff[b] = (uint32_t)(quads.size() / 4);
		b_goff[b] = (uint32_t)ng64;
		body_quads(B, quads);
		b_order[b] = B.quads.empty() ? 2u : B.order;
		uint64_t k = (uint64_t)(quads.size() / 4 - b_eoff[b]) * b_order[b] * b_order[b];
		ng64 += k;
		if (ng64 > 0x7fffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^31 Gauss points");
		gpb.insert(gpb.end(), k, b);
		if (B.gpt[0].empty()) {
			gh.insert(gh.end(), k, B.gp_h);
			grho.insert(grho.end(), k, B.gp_rho);
		} else {
			gh.insert(gh.end(), B.gpt[2].begin(), B.gpt[2].end());
			grho.insert(grho.end(), B.gpt[3].begin(), B.gpt[3].end());
		}
	}
	b_eoff[nb] = (uint32_t)(quads.size() / 4);
	b_goff[nb] = (uint32_t)ng64;
	c->n_g = (uint32_t)ng64;
	uint32_t ng = c->n_g;
	c->do_smooth = c->bodies[0].sd.do_smooth != 0;
	DevBuf<uint32_t> d_quads;
	mf_status st;
	CK(d_quads.alloc(quads.size()));
	CK(cudaMemcpy(d_quads.p, quads.data(), quads.size() * 4, cudaMemcpyHostToDevice));
	CK(c->gp_body.alloc(ng));
	CK(cudaMemcpy(c->gp_body.p, gpb.data(), (size_t)ng * 4, cudaMemcpyHostToDevice));
	CK(c->gp_x.alloc(ng)); CK(c->gp_y.alloc(ng)); CK(c->gp_qw.alloc(ng)); CK(c->gp_hh.alloc(ng));
	CK(c->gp_ux.alloc(ng)); CK(c->gp_uy.alloc(ng));
	CK(cudaMemcpy(c->gp_hh.p, gh.data(), (size_t)ng * 8, cudaMemcpyHostToDevice));
	// update_gauss_points on the reference positions X, body runs of one order per launch
	DevBuf<double> gX, gY, fwx, fwy;
	CK(gX.alloc(ng)); CK(gY.alloc(ng));
	if (fem) { CK(fwx.alloc(4 * (size_t)ng)); CK(fwy.alloc(4 * (size_t)ng)); }
	cudaError_t e = cudaSuccess;
	for (uint32_t b0 = 0, b1; b0 < nb; b0 = b1) {
		for (b1 = b0 + 1; b1 < nb && b_order[b1] == b_order[b0];) b1++;
		const uint32_t eo = b_eoff[b0], go = b_goff[b0], ne = b_eoff[b1] - eo;
		const uint32_t* q = d_quads.p + 4 * (size_t)eo;
		double* w3[3] = {nullptr, fem ? fwx.p + 4 * (size_t)go : nullptr, fem ? fwy.p + 4 * (size_t)go : nullptr};
		e = c->strict ? mf_strict::weak_gauss_points(ne, q, b_order[b0], c->X.p, c->Y.p, gX.p + go, gY.p + go,
		                                             c->gp_qw.p + go, w3[0], w3[1], w3[2], c->d_status, c->stream)
		              : mf_fast::weak_gauss_points(ne, q, b_order[b0], c->X.p, c->Y.p, gX.p + go, gY.p + go,
		                                           c->gp_qw.p + go, w3[0], w3[1], w3[2], c->d_status, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "weak_gauss_points");
	}
	if ((st = check_status(c)) != MF_OK) return st;
	// current Gauss-point positions: as given, else where update_gauss_points put them
	CK(cudaMemcpyAsync(c->gp_x.p, gX.p, (size_t)ng * 8, cudaMemcpyDeviceToDevice, c->stream));
	CK(cudaMemcpyAsync(c->gp_y.p, gY.p, (size_t)ng * 8, cudaMemcpyDeviceToDevice, c->stream));
	for (uint32_t b = 0; b < nb; b++) {
		const HostBody& B = c->bodies[b];
		if (B.gpt[0].empty()) continue;
		CK(cudaMemcpyAsync(c->gp_x.p + b_goff[b], B.gpt[0].data(), B.gpt[0].size() * 8, cudaMemcpyHostToDevice, c->stream));
		CK(cudaMemcpyAsync(c->gp_y.p + b_goff[b], B.gpt[1].data(), B.gpt[1].size() * 8, cudaMemcpyHostToDevice, c->stream));
	}
	e = c->strict ? mf_strict::weak_gp_disp(ng, c->gp_x.p, c->gp_y.p, gX.p, gY.p, c->gp_ux.p, c->gp_uy.p, c->stream)
	              : mf_fast::weak_gp_disp(ng, c->gp_x.p, c->gp_y.p, gX.p, gY.p, c->gp_ux.p, c->gp_uy.p, c->stream);
	if (e != cudaSuccess) return cuda_fail(c, e, "weak_gp_disp");
	CK(cudaStreamSynchronize(c->stream));
	gX.free(); gY.free();
	const double* px = c->sd[0][0].p;
	const double* py = c->sd[0][1].p;

	// lists: Gauss points -> particles, particles -> particles, particles -> Gauss points
	DevBuf<uint32_t> g_off, g_nbr, t_off, t_nbr;
	std::vector<uint32_t> gc, pc, tc;
	DevBuf<double> gwx, gwy, pw, twx, twy;
	if (fem) {
		// the elements' own functions: a Gauss point sees its element's nodes in node order
		// (gauss_integration.h:110-116); the particles have no lists (the *_fem set-ups run
		// no neighbour search); the transposed lists keep the Gauss points ascending, the
		// order of the scatter in derive_stress_weak_tl (derivatives.h:260-294)
		std::vector<uint32_t> goff(ng + 1), gn(4 * (size_t)ng), toff(n + 1, 0), tn(4 * (size_t)ng), tsrc(4 * (size_t)ng);
		for (uint32_t b = 0; b < nb; b++) {
			const uint32_t npe = b_order[b] * b_order[b];
			for (uint32_t g = b_goff[b]; g < b_goff[b + 1]; g++) {
				const uint32_t el = b_eoff[b] + (g - b_goff[b]) / npe;
				for (int k = 0; k < 4; k++) gn[4 * (size_t)g + k] = quads[4 * (size_t)el + k];
			}
		}
		for (uint32_t g = 0; g <= ng; g++) goff[g] = 4 * g;
		for (uint32_t v : gn) toff[v + 1]++;
		tc.assign(toff.begin() + 1, toff.end());
		for (uint32_t j = 0; j < n; j++) toff[j + 1] += toff[j];
		std::vector<uint32_t> pos(toff.begin(), toff.end() - 1);
		for (size_t k = 0; k < gn.size(); k++) {
			uint32_t t = pos[gn[k]]++;
			tn[t] = (uint32_t)(k / 4);
			tsrc[t] = (uint32_t)k;
		}
		gc.assign(ng, 4);
		pc.assign(n, 0);
		std::vector<double> hx(4 * (size_t)ng), hy(4 * (size_t)ng), tx(4 * (size_t)ng), ty(4 * (size_t)ng);
		CK(cudaMemcpy(hx.data(), fwx.p, hx.size() * 8, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(hy.data(), fwy.p, hy.size() * 8, cudaMemcpyDeviceToHost));
		for (size_t t = 0; t < tn.size(); t++) { tx[t] = hx[tsrc[t]]; ty[t] = hy[tsrc[t]]; }
		auto upu = [&](DevBuf<uint32_t>& d, const std::vector<uint32_t>& v) -> mf_status {
			CK(d.alloc(v.size()));
			if (!v.empty()) CK(cudaMemcpy(d.p, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
			return MF_OK;
		};
		auto upd = [&](DevBuf<double>& d, const std::vector<double>& v) -> mf_status {
			CK(d.alloc(v.size()));
			if (!v.empty()) CK(cudaMemcpy(d.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
			return MF_OK;
		};
		std::vector<uint32_t> zoff(n + 1, 0);
		if ((st = upu(g_off, goff)) || (st = upu(g_nbr, gn)) || (st = upu(t_off, toff)) || (st = upu(t_nbr, tn)) ||
		    (st = upu(c->nbr_off, zoff)) || (st = upu(c->nbr, {})) || (st = upd(twx, tx)) || (st = upd(twy, ty)))
			return st;
		CK(pw.alloc(0));
		gwx = fwx; gwy = fwy;
		fwx.p = fwy.p = nullptr;
	} else {
		if ((st = build_lists(c, px, py, c->body_of.p, n, c->gp_x.p, c->gp_y.p, c->gp_body.p, ng, c->cfg.max_nbh, g_off,
		                      g_nbr, gc, false)))
			return st;
		if ((st = build_lists(c, px, py, c->body_of.p, n, px, py, c->body_of.p, n, c->cfg.max_nbh, c->nbr_off, c->nbr, pc,
		                      false)))
			return st;
		if ((st = build_lists(c, c->gp_x.p, c->gp_y.p, c->gp_body.p, ng, px, py, c->body_of.p, n, 8 * c->cfg.max_nbh,
		                      t_off, t_nbr, tc, false)))
			return st;
		uint64_t eg = g_nbr.n, ep = c->nbr.n, et = t_nbr.n;
		// RKPM shape functions, FP64
		CK(gwx.alloc(eg)); CK(gwy.alloc(eg)); CK(pw.alloc(ep)); CK(twx.alloc(et)); CK(twy.alloc(et));
		DevBuf<double> rho_tmp;  // the mixed form keeps no FP64 density; the set-up needs one
		if (c->mixed) {
			CK(rho_tmp.alloc(n));
			std::vector<double> v(n);
			for (auto& b : c->bodies) std::copy(b.in[5].begin(), b.in[5].end(), v.begin() + b.off);
			CK(cudaMemcpy(rho_tmp.p, v.data(), (size_t)n * 8, cudaMemcpyHostToDevice));
		}
		const double* rho64 = c->mixed ? rho_tmp.p : c->sd[0][4].p;
		const float* rho32 = nullptr;
		auto rkpm = [&](uint32_t nt, const double* tx, const double* ty, const double* th, const uint32_t* off,
		                const uint32_t* nbr, double* w, double* wx, double* wy) {
			return c->strict ? mf_strict::weak_rkpm(nt, tx, ty, th, off, nbr, px, py, c->m.p, rho64, rho32, w, wx, wy,
			                                        c->d_status, c->stream)
			                 : mf_fast::weak_rkpm(nt, tx, ty, th, off, nbr, px, py, c->m.p, rho64, rho32, w, wx, wy,
			                                      c->d_status, c->stream);
		};
		if ((e = rkpm(ng, c->gp_x.p, c->gp_y.p, c->gp_hh.p, g_off.p, g_nbr.p, nullptr, gwx.p, gwy.p)) != cudaSuccess)
			return cuda_fail(c, e, "weak_rkpm");
		if ((e = rkpm(n, px, py, c->h.p, c->nbr_off.p, c->nbr.p, pw.p, nullptr, nullptr)) != cudaSuccess)
			return cuda_fail(c, e, "weak_rkpm");
		e = c->strict ? mf_strict::weak_transpose(n, t_off.p, t_nbr.p, g_off.p, g_nbr.p, gwx.p, gwy.p, twx.p, twy.p,
		                                          c->d_status, c->stream)
		              : mf_fast::weak_transpose(n, t_off.p, t_nbr.p, g_off.p, g_nbr.p, gwx.p, gwy.p, twx.p, twy.p,
		                                        c->d_status, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "weak_transpose");
		if ((st = check_status(c)) != MF_OK) return st;
		CK(cudaStreamSynchronize(c->stream));
		rho_tmp.free();
	}
	// sliced ELL (mixed: FP32 with the quad weights folded in)
	uint64_t sg, sp, stt;
	c->g_entries = 0;
	c->t_entries = 0;
	for (uint32_t v : gc) c->g_entries += v;
	for (uint32_t v : tc) c->t_entries += v;
	if ((st = sell_offsets(c, gc, c->g_sl, sg)) || (st = sell_offsets(c, pc, c->p_sl, sp)) ||
	    (st = sell_offsets(c, tc, c->t_sl, stt)))
		return st;
	CK(c->g_cnt.alloc(ng)); CK(c->p_cnt.alloc(n)); CK(c->t_cnt.alloc(n));
	CK(c->g_snbr.alloc(sg)); CK(c->p_snbr.alloc(sp)); CK(c->t_snbr.alloc(stt));
	if (c->mixed) {
		CK(c->g_w32.alloc(sg)); CK(c->p_w32.alloc(sp)); CK(c->t_w32.alloc(stt));
	} else {
		CK(c->g_w64.alloc(sg)); CK(c->p_w64.alloc(sp)); CK(c->t_w64.alloc(stt));
	}
	auto sell = [&](uint32_t nr, const uint32_t* off, const uint32_t* nbr, const double* a, const double* b,
	                const uint32_t* sl, uint16_t* cnt, uint32_t* snbr, void* o64, void* o32, const double* mr,
	                const double* mn) {
		return c->strict ? mf_strict::weak_sell(nr, off, nbr, a, b, sl, cnt, snbr, o64, o32, mr, mn, c->stream)
		                 : mf_fast::weak_sell(nr, off, nbr, a, b, sl, cnt, snbr, o64, o32, mr, mn, c->stream);
	};
	bool mx = c->mixed;
	if ((e = sell(ng, g_off.p, g_nbr.p, gwx.p, gwy.p, c->g_sl.p, c->g_cnt.p, c->g_snbr.p, mx ? nullptr : c->g_w64.p,
	              mx ? (void*)c->g_w32.p : nullptr, nullptr, c->qw0.p)) != cudaSuccess ||
	    (e = sell(n, c->nbr_off.p, c->nbr.p, pw.p, nullptr, c->p_sl.p, c->p_cnt.p, c->p_snbr.p, mx ? nullptr : c->p_w64.p,
	              mx ? (void*)c->p_w32.p : nullptr, nullptr, c->qw0.p)) != cudaSuccess ||
	    (e = sell(n, t_off.p, t_nbr.p, twx.p, twy.p, c->t_sl.p, c->t_cnt.p, c->t_snbr.p, mx ? nullptr : c->t_w64.p,
	              mx ? (void*)c->t_w32.p : nullptr, c->qw0.p, c->gp_qw.p)) != cudaSuccess)
		return cuda_fail(c, e, "weak_sell");
	CK(cudaStreamSynchronize(c->stream));
	gwx.free(); gwy.free(); pw.free(); twx.free(); twy.free(); g_off.free(); g_nbr.free(); t_off.free(); t_nbr.free();
	// Gauss-point state: rho = the set-up rho (tensile.cpp:792-795), S = 0
	// (grho: gp_rho, or the given Gauss-point rho)
	for (int k = 0; k < 3; k++)
		for (int q = 0; q < 4; q++) {
			if (mx) {
				CK(c->gsf[k][q].alloc(ng));
				if (q == 0) {
					std::vector<float> f(ng);
					for (uint32_t g = 0; g < ng; g++) f[g] = (float)(grho[g] - c->bodies[gpb[g]].sd.rho0);
					CK(cudaMemcpy(c->gsf[k][q].p, f.data(), (size_t)ng * 4, cudaMemcpyHostToDevice));
				} else {
					CK(cudaMemset(c->gsf[k][q].p, 0, (size_t)ng * 4));
				}
			} else {
				CK(c->gsd[k][q].alloc(ng));
				if (q == 0) CK(cudaMemcpy(c->gsd[k][q].p, grho.data(), (size_t)ng * 8, cudaMemcpyHostToDevice));
				else CK(cudaMemset(c->gsd[k][q].p, 0, (size_t)ng * 8));
			}
		}
	if (mx) {
		CK(c->gP32.alloc(ng));
		CK(c->wpack.alloc(2 * (size_t)n));
	} else {
		CK(c->gP64.alloc(4 * (size_t)ng));
	}
	// particles: stage 0 starts from a copy of the particles (set 2)
	for (int q = 0; q < 8; q++) {
		if (c->mixed && q >= 4) continue;
		CK(cudaMemcpy(c->sd[2][q].p, c->sd[0][q].p, (size_t)n * 8, cudaMemcpyDeviceToDevice));
	}
	return upload_bcs(c);
}


WeakArgs weak_args(mf_ctx* c) {
	WeakArgs a{};
	a.n_p = c->n_total; a.n_g = c->n_g; a.n_bodies = (uint32_t)c->bodies.size(); a.flags = c->flags;
	a.block = c->tune.tl_block;
	a.params = c->params.p; a.body_of = c->body_of.p; a.gp_body = c->gp_body.p;
	a.X = c->X.p; a.Y = c->Y.p; a.m = c->m.p; a.qw_p = c->qw0.p; a.gp_qw = c->gp_qw.p; a.fcx = c->fcx.p; a.fcy = c->fcy.p;
	a.gp_ux = c->gp_ux.p; a.gp_uy = c->gp_uy.p;
	StateSoA* s[3] = {&a.base, &a.acc, &a.st};
	for (int k = 0; k < 3; k++) {
		double** d[8] = {&s[k]->x, &s[k]->y, &s[k]->vx, &s[k]->vy, &s[k]->rho, &s[k]->Sxx, &s[k]->Sxy, &s[k]->Syy};
		for (int q = 0; q < 8; q++) *d[q] = c->sd[k][q].p;
	}
	StateSoA* g[3] = {&a.gbase, &a.gacc, &a.gst};
	for (int k = 0; k < 3; k++) {
		g[k]->rho = c->gsd[k][0].p; g[k]->Sxx = c->gsd[k][1].p; g[k]->Sxy = c->gsd[k][2].p; g[k]->Syy = c->gsd[k][3].p;
		g[k]->rho_f = c->gsf[k][0].p; g[k]->Sxx_f = c->gsf[k][1].p; g[k]->Sxy_f = c->gsf[k][2].p; g[k]->Syy_f = c->gsf[k][3].p;
	}
	a.g_sl = c->g_sl.p; a.g_snbr = c->g_snbr.p; a.g_cnt = c->g_cnt.p;
	a.t_sl = c->t_sl.p; a.t_snbr = c->t_snbr.p; a.t_cnt = c->t_cnt.p;
	a.p_sl = c->p_sl.p; a.p_snbr = c->p_snbr.p; a.p_cnt = c->p_cnt.p;
	a.g_w = c->mixed ? (const void*)c->g_w32.p : (const void*)c->g_w64.p;
	a.t_w = c->mixed ? (const void*)c->t_w32.p : (const void*)c->t_w64.p;
	a.p_w = c->mixed ? (const void*)c->p_w32.p : (const void*)c->p_w64.p;
	a.gP = c->mixed ? (void*)c->gP32.p : (void*)c->gP64.p;
	a.pack = c->wpack.p;
	a.bc_rows = c->bc_rows.p; a.bc_v = c->bc_v.p; a.n_bc = c->n_bc;
	a.status = c->d_status;
	return a;
}

// rk4::do_step_weak + step for particle_tl_weak (rk4.h:140-185, 207-218): four stages
// of (BCs, Gauss-point pass, particle pass), then the clock, the BCs on the particles
// and the velocity smoothing -- in the reference's order.
mf_status weak_step(mf_ctx* c) {
	WeakArgs a = weak_args(c);
	auto launch = [&](int part) {
		return c->strict ? mf_strict::weak_stage(a, c->mixed, part, c->stream)
		                 : mf_fast::weak_stage(a, c->mixed, part, c->stream);
	};
	cudaError_t e;
	for (uint32_t st = 0; st < 4; st++) {
		a.stage = st;
		if ((e = launch(0)) != cudaSuccess || (e = launch(1)) != cudaSuccess) return cuda_fail(c, e, "weak stage");
		int slot;
		timing_begin(c, 5, slot);
		if ((e = launch(2)) != cudaSuccess) return cuda_fail(c, e, "weak Gauss-point pass");
		timing_end(c, slot, c->n_g);
		timing_begin(c, 2, slot);
		if ((e = launch(3)) != cudaSuccess) return cuda_fail(c, e, "weak particle pass");
		timing_end(c, slot, c->n_total);
		c->launches += 2 + (c->n_bc ? 1 : 0) + (c->mixed ? 1 : 0);
	}
	if ((e = launch(6)) != cudaSuccess || (e = launch(4)) != cudaSuccess) return cuda_fail(c, e, "weak step end");
	c->launches += 1 + (c->n_bc ? 1 : 0);
	if (c->do_smooth) {
		if ((e = launch(5)) != cudaSuccess) return cuda_fail(c, e, "weak smoothing");
		c->launches += 2;
	}
	return MF_OK;
}

// Weak updated-Lagrangian pipeline: a subsequence, in this order, of the reference's
// list (tensile.cpp:713-726; rings.cpp:917-930 with the mass-divided momentum), with
// the data dependencies present.  Ids 35-40 take the FLAG_UW_* bits.
mf_status validate_ulweak(mf_ctx* c, const std::vector<int32_t>& acts, uint32_t& flags) {
	static const int order[] = {MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS, MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP,
	                            MF_MATERIAL_EOS_GP, MF_DERIVE_STRESS_WEAK_UL, MF_DERIVE_VELOCITY_WEAK, MF_DERIVE_VELOCITY,
	                            MF_MATERIAL_STRESS_RATE_JAUMANN_GP, MF_CONTMECH_MOMENTUM_UL, MF_CONTMECH_MOMENTUM_UL_WEAK,
	                            MF_CONTMECH_CONTINUITY, MF_CONTMECH_CONTINUITY_GP, MF_CONTMECH_ADVECTION,
	                            MF_INTERPOLATION_INTERPOLATE_VELOCITY, MF_CONTMECH_ADVECTION_GP};
	flags = 0;
	size_t pos = 0;
	for (int32_t a : acts) {
		while (pos < sizeof(order) / sizeof(order[0]) && order[pos] != a) pos++;
		if (pos == sizeof(order) / sizeof(order[0]))
			return fail(c, MF_ERR_PIPELINE, "action %d is not part of the weak UL pipeline or out of its order", a);
		pos++;
		switch (a) {
		case MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP: flags |= FLAG_UW_RIEMANN_GP; break;
		case MF_DERIVE_STRESS_WEAK_UL: flags |= FLAG_UW_STRESS; break;
		case MF_DERIVE_VELOCITY_WEAK: flags |= FLAG_UW_VEL_WEAK; break;
		case MF_CONTMECH_MOMENTUM_UL_WEAK: flags |= FLAG_UW_MOMENTUM_W; break;
		case MF_INTERPOLATION_INTERPOLATE_VELOCITY: flags |= FLAG_UW_INTERP; break;
		case MF_CONTMECH_ADVECTION_GP: flags |= FLAG_UW_ADVECTION_GP; break;
		default: flags |= abit(a);
		}
	}
	const bool mom = (flags & abit(MF_CONTMECH_MOMENTUM_UL)) || (flags & FLAG_UW_MOMENTUM_W);
	if ((flags & abit(MF_CONTMECH_MOMENTUM_UL)) && (flags & FLAG_UW_MOMENTUM_W))
		return fail(c, MF_ERR_PIPELINE, "contmech_momentum_ul and contmech_momentum_ul_weak both add the stress forces");
	if (mom && !(flags & FLAG_UW_STRESS))
		return fail(c, MF_ERR_PIPELINE, "the momentum needs derive_stress_weak_ul before it");
	if ((flags & (abit(MF_MATERIAL_STRESS_RATE_JAUMANN_GP) | abit(MF_CONTMECH_CONTINUITY_GP))) &&
	    !(flags & FLAG_UW_VEL_WEAK))
		return fail(c, MF_ERR_PIPELINE, "the stress points' Jaumann rate / continuity need derive_velocity_weak");
	if ((flags & abit(MF_CONTMECH_CONTINUITY)) && !(flags & abit(MF_DERIVE_VELOCITY)))
		return fail(c, MF_ERR_PIPELINE, "contmech_continuity needs derive_velocity before it");
	if ((flags & FLAG_UW_ADVECTION_GP) && !(flags & FLAG_UW_INTERP))
		return fail(c, MF_ERR_PIPELINE, "contmech_advection_gp needs interpolation_interpolate_velocity before it");
	if ((flags & abit(MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS)) && !c->bodies.empty() && !c->bodies[0].quads.empty())
		return fail(c, MF_ERR_PIPELINE, "riemann_update_integration_weights runs with the ellipse (no element maps)");
	return MF_OK;
}

// CSR lists (off, nbr) of n rows laid out in slices of 32 rows: the k-th candidate of
// row i in slot base(i / 32) + 32 k + i % 32, each slice as wide as its longest row.
// Gives the rows' first slots and counts and the sliced list (slots past a row's count
// are padding, never read); false when the slots do not fit 32-bit indices.
bool slice_lists(const std::vector<uint32_t>& off, const std::vector<uint32_t>& nbr, uint32_t n,
                 std::vector<uint32_t>& start, std::vector<uint32_t>& cnt, std::vector<uint32_t>& sliced) {
	start.assign((size_t)n + 1, 0);
	cnt.assign((size_t)n + 1, 0);
	uint64_t base = 0;
	for (uint32_t s0 = 0; s0 < n; s0 += 32) {
		const uint32_t s1 = std::min(n, s0 + 32);
		uint32_t width = 0;
		for (uint32_t i = s0; i < s1; i++) width = std::max(width, off[i + 1] - off[i]);
		for (uint32_t i = s0; i < s1; i++) {
			start[i] = (uint32_t)(base + (i - s0));
			cnt[i] = off[i + 1] - off[i];
		}
		base += 32ull * width;
		if (base >= 0xffffffffull) return false;
	}
	sliced.assign(base, 0);
	for (uint32_t i = 0; i < n; i++)
		for (uint32_t k = 0; k < cnt[i]; k++) sliced[start[i] + 32ull * k] = nbr[off[i] + k];
	return true;
}

// Weak UL set-up: stress points, candidate lists by the Manhattan search
// (tensile.cpp:706-707), the transposed stress-point candidates, per-candidate scratch.
mf_status uw_setup(mf_ctx* c) {
	const uint32_t n = c->n_total;
	// a gauss_int in place of the ellipse (body.h:91-99): every body on an element map
	const bool fem = !c->bodies[0].quads.empty();
	if (!fem && !(c->cfg.nbh_h > 0.))
		return fail(c, MF_ERR_ARG, "the weak UL form needs config.nbh_h > 0 (the candidate search h)");
	uint32_t ng = 0;
	for (auto& b : c->bodies) {
		if (b.n_sp == 0) return fail(c, MF_ERR_STATE, "a UL_WEAK body needs mf_set_stress_points");
		if (b.quads.empty() == fem || (fem && b.order != c->bodies[0].order))
			return fail(c, MF_ERR_PIPELINE, "UL_WEAK bodies take all the ellipse or all element maps of one order");
		if (fem && (uint64_t)b.order * b.order * (b.quads.size() / 4) != b.n_sp)
			return fail(c, MF_ERR_ARG, "a UL_WEAK element map of %zu elements needs %u stress points per element",
			            b.quads.size() / 4, b.order * b.order);
		ng += b.n_sp;
	}
	if (fem && c->bodies[0].sd.do_smooth)
		return fail(c, MF_ERR_PIPELINE, "velocity smoothing needs the ellipse neighbourhoods (no element maps)");
	c->n_g = ng;
	c->do_smooth = c->bodies[0].sd.do_smooth != 0;
	std::vector<uint32_t> gb(ng);
	std::vector<double> gv[13];
	for (int k = 0; k < 13; k++) gv[k].reserve(ng);
	for (size_t b = 0, o = 0; b < c->bodies.size(); b++) {
		const HostBody& B = c->bodies[b];
		for (uint32_t i = 0; i < B.n_sp; i++) gb[o++] = (uint32_t)b;
		for (int k = 0; k < 13; k++) gv[k].insert(gv[k].end(), B.sp[k].begin(), B.sp[k].end());
	}
	auto up = [&](DevBuf<double>& d, const std::vector<double>& v) -> mf_status {
		CK(d.alloc(v.size()));
		CK(cudaMemcpy(d.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
		return MF_OK;
	};
	mf_status st;
	CK(c->uw_gbody.alloc(ng));
	CK(cudaMemcpy(c->uw_gbody.p, gb.data(), (size_t)ng * 4, cudaMemcpyHostToDevice));
	// stress-point state: x y rho Sxx Sxy Syy (input fields 0 1 5 10 11 12)
	const int gf[6] = {0, 1, 5, 10, 11, 12};
	for (int q = 0; q < 6; q++) {
		if ((st = up(c->uw_g[0][q], gv[gf[q]]))) return st;
		for (int k = 1; k < 4; k++) CK(c->uw_g[k][q].alloc(ng));
	}
	if ((st = up(c->uw_gm, gv[4])) || (st = up(c->uw_gqw, gv[7]))) return st;
	CK(c->uw_gh.alloc(ng)); CK(c->uw_gsig.alloc(4 * (size_t)ng));
	// particles: the weights of the last riemann update (the input weights at first)
	CK(c->uw_qwp.alloc(n));
	CK(cudaMemcpy(c->uw_qwp.p, c->qw0.p, (size_t)n * 8, cudaMemcpyDeviceToDevice));
	CK(c->uw_ph.alloc(n)); CK(c->uw_qws.alloc(n));
	if (c->uw_mixed) {
		CK(c->uw_ff.alloc(4 * (size_t)n)); CK(c->uw_vol.alloc(n));
		CK(c->uw_vff.alloc(4 * (size_t)n)); CK(c->uw_qw32.alloc(n)); CK(c->uw_qwlo.alloc(n));
		CK(c->uw_gsig32.alloc(4 * (size_t)ng));
	}
	for (int q = 0; q < 8; q++) CK(c->sd[3][q].alloc(n));
	std::vector<uint32_t> goff(ng + 1), gnbr, gstart;
	uint64_t ep, eg;
	if (fem) {
		// the particles have no lists; a stress point's candidates are its element's
		// nodes in node order (gauss_integration.h:110-116), all of them used; the
		// particles' weights stay the input ones (no ellipse, no riemann update)
		std::vector<uint32_t> quads;
		for (auto& b : c->bodies) body_quads(b, quads);
		c->uw_order = c->bodies[0].order;
		c->uw_nelem = (uint32_t)(quads.size() / 4);
		const uint32_t npe = c->uw_order * c->uw_order;
		gnbr.resize(4 * (size_t)ng);
		for (uint32_t g = 0; g < ng; g++)
			for (int k = 0; k < 4; k++) gnbr[4 * (size_t)g + k] = quads[4 * (size_t)(g / npe) + k];
		for (uint32_t g = 0; g <= ng; g++) goff[g] = 4 * g;
		std::vector<uint32_t> zoff(n + 1, 0);
		CK(c->uw_quads.alloc(quads.size()));
		CK(cudaMemcpy(c->uw_quads.p, quads.data(), quads.size() * 4, cudaMemcpyHostToDevice));
		CK(c->uw_pc_off.alloc(n + 1)); CK(c->uw_pc_nbr.alloc(0));
		CK(cudaMemcpy(c->uw_pc_off.p, zoff.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
		CK(c->uw_gc_off.alloc(ng + 1)); CK(c->uw_gc_nbr.alloc(gnbr.size()));
		CK(cudaMemcpy(c->uw_gc_off.p, goff.data(), ((size_t)ng + 1) * 4, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->uw_gc_nbr.p, gnbr.data(), gnbr.size() * 4, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->uw_qws.p, c->qw0.p, (size_t)n * 8, cudaMemcpyDeviceToDevice));
		std::vector<uint32_t> four(ng + 1, 4);
		CK(c->uw_pc_cnt.alloc(n + 1)); CK(c->uw_gc_cnt.alloc(ng + 1));
		CK(cudaMemcpy(c->uw_pc_cnt.p, zoff.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->uw_gc_cnt.p, four.data(), ((size_t)ng + 1) * 4, cudaMemcpyHostToDevice));
		c->uw_pc_stride = c->uw_gc_stride = 1;
		gstart.assign(goff.begin(), goff.end());
		ep = 0;
		eg = gnbr.size();
	} else {
		// candidate lists (CSR, ascending)
		std::vector<uint32_t> pc, gc;
		const double *px = c->sd[0][0].p, *py = c->sd[0][1].p;
		if ((st = build_lists(c, px, py, c->body_of.p, n, px, py, c->body_of.p, n, c->cfg.max_nbh, c->uw_pc_off,
		                      c->uw_pc_nbr, pc, true)))
			return st;
		if ((st = build_lists(c, px, py, c->body_of.p, n, c->uw_g[0][0].p, c->uw_g[0][1].p, c->uw_gbody.p, ng,
		                      c->cfg.max_nbh, c->uw_gc_off, c->uw_gc_nbr, gc, true)))
			return st;
		gnbr.resize(c->uw_gc_nbr.n);
		CK(cudaMemcpy(goff.data(), c->uw_gc_off.p, ((size_t)ng + 1) * 4, cudaMemcpyDeviceToHost));
		if (!gnbr.empty()) CK(cudaMemcpy(gnbr.data(), c->uw_gc_nbr.p, gnbr.size() * 4, cudaMemcpyDeviceToHost));
		std::vector<uint32_t> poff(n + 1), pnbr(c->uw_pc_nbr.n);
		CK(cudaMemcpy(poff.data(), c->uw_pc_off.p, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
		if (!pnbr.empty()) CK(cudaMemcpy(pnbr.data(), c->uw_pc_nbr.p, pnbr.size() * 4, cudaMemcpyDeviceToHost));
		// the ellipse kernels and the passes walk the lists one row per thread: sliced,
		// a warp's 32 rows reach their k-th candidates in one line
		std::vector<uint32_t> pstart, pcnt, psl, gcnt, gsl;
		if (!slice_lists(poff, pnbr, n, pstart, pcnt, psl) || !slice_lists(goff, gnbr, ng, gstart, gcnt, gsl))
			return fail(c, MF_ERR_CAPACITY, "weak UL candidate slots exceed 2^32");
		auto upload = [&](DevBuf<uint32_t>& d, const std::vector<uint32_t>& v) -> mf_status {
			d.free();
			CK(d.alloc(v.size()));
			if (!v.empty()) CK(cudaMemcpy(d.p, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
			return MF_OK;
		};
		if ((st = upload(c->uw_pc_off, pstart)) || (st = upload(c->uw_pc_cnt, pcnt)) || (st = upload(c->uw_pc_nbr, psl)) ||
		    (st = upload(c->uw_gc_off, gstart)) || (st = upload(c->uw_gc_cnt, gcnt)) || (st = upload(c->uw_gc_nbr, gsl)))
			return st;
		c->uw_pc_stride = c->uw_gc_stride = 32;
		ep = psl.size();
		eg = gsl.size();
	}
	CK(c->uw_pmask.alloc(ep)); CK(c->uw_pw.alloc(ep)); CK(c->uw_pwx.alloc(ep)); CK(c->uw_pwy.alloc(ep));
	CK(c->uw_gmask.alloc(eg)); CK(c->uw_gw.alloc(eg)); CK(c->uw_gwx.alloc(eg)); CK(c->uw_gwy.alloc(eg));
	if (fem) CK(cudaMemset(c->uw_gmask.p, 1, eg));
	// per particle, the stress points whose candidates hold it (ascending) and the slot
	const uint64_t et = gnbr.size();  // stress-point candidates (the transposed entries)
	std::vector<uint32_t> toff(n + 1, 0), tgp(et), tslot(et);
	for (uint64_t q = 0; q < et; q++) toff[gnbr[q] + 1]++;
	for (uint32_t j = 0; j < n; j++) toff[j + 1] += toff[j];
	std::vector<uint32_t> fill(toff.begin(), toff.end() - 1);
	for (uint32_t i = 0; i < ng; i++)
		for (uint32_t q = goff[i]; q < goff[i + 1]; q++) {
			uint32_t t = fill[gnbr[q]]++;
			tgp[t] = i;
			tslot[t] = gstart[i] + (q - goff[i]) * c->uw_gc_stride;
		}
	// sliced like the candidate lists (the particle pass walks them one row per thread)
	std::vector<uint32_t> tstart, tcnt, tgp_sl, tslot_sl;
	if (!slice_lists(toff, tgp, n, tstart, tcnt, tgp_sl) || !slice_lists(toff, tslot, n, tstart, tcnt, tslot_sl))
		return fail(c, MF_ERR_CAPACITY, "weak UL transposed slots exceed 2^32");
	CK(c->uw_tp_off.alloc(n + 1)); CK(c->uw_tp_cnt.alloc(n + 1));
	CK(c->uw_tp_gp.alloc(tgp_sl.size())); CK(c->uw_tp_slot.alloc(tslot_sl.size()));
	CK(cudaMemcpy(c->uw_tp_off.p, tstart.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
	CK(cudaMemcpy(c->uw_tp_cnt.p, tcnt.data(), ((size_t)n + 1) * 4, cudaMemcpyHostToDevice));
	if (!tgp_sl.empty()) {
		CK(cudaMemcpy(c->uw_tp_gp.p, tgp_sl.data(), tgp_sl.size() * 4, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->uw_tp_slot.p, tslot_sl.data(), tslot_sl.size() * 4, cudaMemcpyHostToDevice));
	}
	// boundary conditions: the rows' index into the value list
	if ((st = upload_bcs(c))) return st;
	std::vector<uint32_t> bc_of(n, ~0u);
	uint32_t k = 0;
	for (auto& b : c->bodies)
		for (auto& bc : b.bcs)
			for (uint32_t i : bc.idx) bc_of[b.off + i] = k++;
	CK(c->uw_bc_of.alloc(n));
	CK(cudaMemcpy(c->uw_bc_of.p, bc_of.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
	return MF_OK;
}

UWArgs uw_args(mf_ctx* c, uint32_t stage) {
	UWArgs a{};
	a.n_p = c->n_total; a.n_g = c->n_g; a.stage = stage; a.flags = c->flags;
	a.params = c->params.p; a.body_of = c->body_of.p; a.gbody_of = c->uw_gbody.p;
	a.m = c->m.p; a.gm = c->uw_gm.p; a.fcx = c->fcx.p; a.fcy = c->fcy.p;
	a.qw_base = c->uw_qwp.p; a.gqw_base = c->uw_gqw.p; a.qw_stage = c->uw_qws.p;
	auto soa = [&](int k) {
		StateSoA s{};
		s.x = c->sd[k][0].p; s.y = c->sd[k][1].p; s.vx = c->sd[k][2].p; s.vy = c->sd[k][3].p;
		s.rho = c->sd[k][4].p; s.Sxx = c->sd[k][5].p; s.Sxy = c->sd[k][6].p; s.Syy = c->sd[k][7].p;
		return s;
	};
	auto gsoa = [&](int k) {
		GSoA g{c->uw_g[k][0].p, c->uw_g[k][1].p, c->uw_g[k][2].p, c->uw_g[k][3].p, c->uw_g[k][4].p, c->uw_g[k][5].p};
		return g;
	};
	// stage 0 reads the particles themselves (rk4.h:144-150), then sets 2 and 3 alternate
	const int rd = stage == 0 ? 0 : (stage % 2 == 1 ? 2 : 3);
	const int wr = stage % 2 == 0 ? 2 : 3;
	a.base = soa(0); a.acc = soa(1); a.rd = soa(rd); a.wr = soa(wr);
	a.gbase = gsoa(0); a.gacc = gsoa(1); a.grd = gsoa(rd); a.gwr = gsoa(wr);
	a.pc = {c->uw_pc_off.p, c->uw_pc_cnt.p, c->uw_pc_nbr.p, c->uw_pc_stride};
	a.gc = {c->uw_gc_off.p, c->uw_gc_cnt.p, c->uw_gc_nbr.p, c->uw_gc_stride};
	a.pmask = c->uw_pmask.p; a.gmask = c->uw_gmask.p;
	a.pw = c->uw_pw.p; a.pwx = c->uw_pwx.p; a.pwy = c->uw_pwy.p;
	a.gw = c->uw_gw.p; a.gwx = c->uw_gwx.p; a.gwy = c->uw_gwy.p;
	a.tp = {c->uw_tp_off.p, c->uw_tp_cnt.p, c->uw_tp_gp.p, 32};
	a.tp_slot = c->uw_tp_slot.p;
	a.gsig = c->uw_gsig.p; a.bc_of = c->uw_bc_of.p; a.bc_v = c->bc_v.p;
	if (c->uw_mixed && !c->strict && !c->uw_order) {
		a.vff = reinterpret_cast<const float4*>(c->uw_vff.p);
		a.qw32 = c->uw_qw32.p;
		a.qwlo = c->uw_qwlo.p;
		a.gsig32 = reinterpret_cast<float4*>(c->uw_gsig32.p);
	}
	a.status = c->d_status;
	return a;
}

// The ellipse neighbourhoods and shape functions of the particles (and, when
// `points`, of the stress points) at the state `a.rd`.  The particles' weights: with
// `refresh_qw` m / rho into the stored weights (the smoothing's riemann update,
// rk4.h:201), else this evaluation's weights into qw_stage (m / rho when the pipeline
// updates them, the stored ones otherwise).
cudaError_t uw_neighbourhoods(mf_ctx* c, const UWArgs& a, bool points, bool refresh_qw) {
	// the mixed form reads the candidates' positions as float-float pairs
	const bool mixed = c->uw_mixed && !c->strict;
	auto nbh = [&](uint32_t n_to, const double* tx, const double* ty, const mfk_host::SlotList& cand, double* h,
	               uint8_t* mask, double* w, double* wx, double* wy, const double* qs, double* qd) {
		return c->strict ? mf_strict::uw_nbh(n_to, tx, ty, cand, a.rd.x, a.rd.y, a.m, a.rd.rho, h, mask, w, wx, wy,
		                                     qs, qd, nullptr, nullptr, c->d_status, c->stream)
		                 : mf_fast::uw_nbh(n_to, tx, ty, cand, a.rd.x, a.rd.y, a.m, a.rd.rho, h, mask, w, wx, wy, qs,
		                                   qd, mixed ? c->uw_ff.p : nullptr, mixed ? c->uw_vol.p : nullptr,
		                                   c->d_status, c->stream);
	};
	const bool riemann = (c->flags & abit(MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS)) != 0;
	const double* qs = refresh_qw ? nullptr : (riemann ? nullptr : a.qw_base);
	double* qd = refresh_qw ? a.qw_base : a.qw_stage;
	if (mixed) {  // the particles' weights come with the float-float inputs
		cudaError_t e = mf_fast::uw_ff(a.n_p, a.rd.x, a.rd.y, a.rd.vx, a.rd.vy, a.m, a.rd.rho, qs, qd, c->uw_ff.p,
		                               c->uw_vff.p, c->uw_vol.p, c->uw_qw32.p, c->uw_qwlo.p, c->stream);
		if (e != cudaSuccess) return e;
		c->launches++;
		qs = nullptr;
		qd = nullptr;
	}
	cudaError_t e = nbh(a.n_p, a.rd.x, a.rd.y, a.pc, c->uw_ph.p, a.pmask, a.pw, a.pwx, a.pwy, qs, qd);
	if (e == cudaSuccess && points)
		e = nbh(a.n_g, a.grd.x, a.grd.y, a.gc, c->uw_gh.p, a.gmask, a.gw, a.gwx, a.gwy, nullptr, nullptr);
	return e;
}

// rk4::do_step_weak + step for particle_ul_weak (rk4.h:140-205): per stage the
// neighbourhoods and shape functions, the stress-point pass, the particle pass; then
// the velocity conditions and the smoothing with fresh neighbourhoods.
mf_status uw_step(mf_ctx* c) {
	cudaError_t e;
	auto launch = [&](const UWArgs& a, int part) {
		return c->strict ? mf_strict::uw_stage(a, part, c->stream) : mf_fast::uw_stage(a, part, c->stream);
	};
	for (uint32_t st = 0; st < 4; st++) {
		UWArgs a = uw_args(c, st);
		if (c->uw_order) {
			// update_gauss_points on this stage's nodes (body.h:97): weights J w and the
			// element functions into the stress points' candidate slots
			e = c->strict ? mf_strict::weak_gauss_points(c->uw_nelem, c->uw_quads.p, c->uw_order, a.rd.x, a.rd.y, nullptr,
			                                             nullptr, c->uw_gqw.p, c->uw_gw.p, c->uw_gwx.p, c->uw_gwy.p,
			                                             c->d_status, c->stream)
			              : mf_fast::weak_gauss_points(c->uw_nelem, c->uw_quads.p, c->uw_order, a.rd.x, a.rd.y, nullptr,
			                                           nullptr, c->uw_gqw.p, c->uw_gw.p, c->uw_gwx.p, c->uw_gwy.p,
			                                           c->d_status, c->stream);
			if (e != cudaSuccess) return cuda_fail(c, e, "weak UL Gauss points");
			c->launches++;
		} else {
			int slot;
			timing_begin(c, 6, slot);
			if ((e = uw_neighbourhoods(c, a, true, false)) != cudaSuccess) return cuda_fail(c, e, "weak UL neighbourhoods");
			timing_end(c, slot, (uint64_t)c->n_total + c->n_g);
		}
		int slot;
		timing_begin(c, 5, slot);
		if ((e = launch(a, 0)) != cudaSuccess) return cuda_fail(c, e, "weak UL stress-point pass");
		timing_end(c, slot, c->n_g);
		timing_begin(c, 2, slot);
		if ((e = launch(a, 1)) != cudaSuccess) return cuda_fail(c, e, "weak UL particle pass");
		timing_end(c, slot, c->n_total);
		c->launches += 4;
	}
	if (c->n_bc) {  // rk4.h:196
		e = c->strict ? mf_strict::ul_bc(c->n_bc, c->bc_rows.p, c->bc_v.p, c->sd[0][2].p, c->sd[0][3].p, c->stream)
		              : mf_fast::ul_bc(c->n_bc, c->bc_rows.p, c->bc_v.p, c->sd[0][2].p, c->sd[0][3].p, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "weak UL conditions");
		c->launches++;
	}
	if (c->do_smooth) {  // rk4.h:198-204
		UWArgs a = uw_args(c, 0);  // reads the particles themselves
		int slot;
		timing_begin(c, 6, slot);
		if ((e = uw_neighbourhoods(c, a, false, true)) != cudaSuccess) return cuda_fail(c, e, "weak UL smoothing");
		timing_end(c, slot, c->n_total);
		if ((e = launch(a, 2)) != cudaSuccess || (e = launch(a, 3)) != cudaSuccess)
			return cuda_fail(c, e, "weak UL smoothing");
		c->launches += 3;
	}
	return MF_OK;
}

// Contact set-up: boundary points, 32-point tiles, and for every body with a
// boundary its master -- the last other body of its group with a boundary, since
// main() loops over ordered pairs and each call first zeroes the slave's forces
// (mfree_iwf.cpp:91-97, contact.h:50-53).
mf_status contact_setup(mf_ctx* c) {
	uint32_t nb = (uint32_t)c->bodies.size();
	std::vector<uint32_t> rows, bstart, blen, tfirst, tend, srows, smaster, mtoff(nb, 0), mtn(nb, 0);
	std::vector<double> sdt;
	for (uint32_t b = 0; b < nb; b++) {
		const HostBody& B = c->bodies[b];
		uint32_t start = (uint32_t)rows.size();
		mtoff[b] = (uint32_t)tfirst.size();
		for (uint32_t i = 0; i < B.hull.size(); i++) {
			rows.push_back(B.off + B.hull[i]);
			bstart.push_back(start);
			blen.push_back((uint32_t)B.hull.size());
		}
		for (uint32_t t = 0; t < B.hull.size(); t += 32) {
			tfirst.push_back(start + t);
			tend.push_back(start + std::min<uint32_t>(t + 32, (uint32_t)B.hull.size()));
		}
		mtn[b] = (uint32_t)tfirst.size() - mtoff[b];
	}
	if (c->cfg.contact) {
		for (uint32_t j = 0; j < nb; j++) {
			if (c->bodies[j].hull.empty()) continue;
			int master = -1;
			for (uint32_t i = 0; i < nb; i++)
				if (i != j && !c->bodies[i].hull.empty() && c->bodies[i].group == c->bodies[j].group) master = (int)i;
			if (master < 0) continue;
			// the body's queries along a Morton curve of the set-up positions (cells of one
			// smoothing length): a warp's 32 queries form a compact patch, so the master
			// tiles that can hold their nearest points are few (a column of 32 rows would
			// span 32 lattice spacings); each query writes only its own row's force, so the
			// order changes no result
			const HostBody& S = c->bodies[j];
			std::vector<std::pair<uint32_t, uint32_t>> order(S.n);
			double x0 = 0., y0 = 0., hcell = 1.;
			if (S.n) {
				x0 = *std::min_element(S.in[0].begin(), S.in[0].end());
				y0 = *std::min_element(S.in[1].begin(), S.in[1].end());
				hcell = S.in[6][0] > 0. ? S.in[6][0] : 1.;
			}
			for (uint32_t r = 0; r < S.n; r++) {
				const double fx = std::floor((S.in[0][r] - x0) / hcell), fy = std::floor((S.in[1][r] - y0) / hcell);
				const uint32_t ix = (uint32_t)std::min(std::max(fx, 0.), 65535.), iy = (uint32_t)std::min(std::max(fy, 0.), 65535.);
				order[r] = {morton_spread(ix) | (morton_spread(iy) << 1), r};
			}
			std::stable_sort(order.begin(), order.end(),
			                 [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
				                 return a.first < b.first;
			                 });
			for (const auto& o : order) {
				srows.push_back(S.off + o.second);
				smaster.push_back((uint32_t)master);
				sdt.push_back(S.dt);
			}
		}
	}
	c->n_bnd = (uint32_t)rows.size();
	c->n_tiles = (uint32_t)tfirst.size();
	c->n_slave = (uint32_t)srows.size();
	c->contact_on = c->cfg.contact && c->n_slave > 0;
	if (!c->contact_on) return MF_OK;
	if (!c->side) {  // for the contact query beside pass A (contact_deferred)
		CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
		CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
		CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
	}
	auto up = [&](DevBuf<uint32_t>& d, const std::vector<uint32_t>& v) -> mf_status {
		CK(d.alloc(v.size()));
		if (!v.empty()) CK(cudaMemcpy(d.p, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
		return MF_OK;
	};
	mf_status st;
	if ((st = up(c->bnd_rows, rows)) || (st = up(c->bnd_start, bstart)) || (st = up(c->bnd_len, blen)) ||
	    (st = up(c->tile_first, tfirst)) || (st = up(c->tile_end, tend)) || (st = up(c->slave_rows, srows)) ||
	    (st = up(c->slave_master, smaster)) || (st = up(c->m_tile_off, mtoff)) || (st = up(c->m_tile_n, mtn)))
		return st;
	CK(c->slave_dt.alloc(sdt.size()));
	CK(cudaMemcpy(c->slave_dt.p, sdt.data(), sdt.size() * 8, cudaMemcpyHostToDevice));
	CK(c->bnd.alloc(c->n_bnd));
	CK(c->bnd_ff.alloc(c->n_bnd));
	CK(c->tile_bb.alloc(c->n_tiles));
	return MF_OK;
}

mf_status contact_run(mf_ctx* c, cudaStream_t s) {
	ContactArgs a{};
	a.n_bnd = c->n_bnd; a.n_tiles = c->n_tiles; a.n_slave = c->n_slave;
	a.bnd_rows = c->bnd_rows.p; a.bnd_start = c->bnd_start.p; a.bnd_len = c->bnd_len.p;
	a.bnd = c->bnd.p; a.bnd_ff = c->bnd_ff.p; a.tile_first = c->tile_first.p; a.tile_end = c->tile_end.p; a.tile_bb = c->tile_bb.p;
	a.slave_rows = c->slave_rows.p; a.slave_master = c->slave_master.p; a.dt = c->slave_dt.p;
	a.m_tile_off = c->m_tile_off.p; a.m_tile_n = c->m_tile_n.p;
	a.x = c->sd[0][0].p; a.y = c->sd[0][1].p; a.m = c->m.p; a.fcx = c->fcx.p; a.fcy = c->fcy.p;
	int slot = -1;
	if (s == c->stream) timing_begin(c, 3, slot);
	cudaError_t e = c->strict ? mf_strict::contact_step(a, s) : mf_fast::contact_step(a, s);
	timing_end(c, slot, c->n_slave);
	if (e != cudaSuccess) return cuda_fail(c, e, "contact");
	c->launches += 3;
	return MF_OK;
}

// Mixed TL with contact: the contact query of the positions a step ends with is left
// pending and runs at the start of the next step on a side stream, beside stage 0's
// pass A (which reads no contact force); pass B waits for it.  The same kernels on the
// same positions, so the same results: only when the forces are computed moves.  Off
// with the monitor (it reads the forces at the end of every step) and with per-kernel
// timing.
bool contact_deferred(const mf_ctx* c) {
	return c->contact_on && c->contact_overlap && c->cfg.method == MF_METHOD_TL && c->mixed && !c->mon_cap &&
	       !c->timing.on;
}

// Runs a pending contact query now (before anything reads the forces or replaces the
// positions it belongs to).
mf_status contact_flush(mf_ctx* c) {
	if (!c->contact_pending) return MF_OK;
	c->contact_pending = false;
	CK(cudaSetDevice(c->cfg.device));
	return contact_run(c, c->stream);
}

}  // namespace

mf_ctx::~mf_ctx() {
	if (io_thread.joinable()) io_thread.join();
	for (cudaStream_t xs : {xs_d2h, xs_h2d})
		if (xs) {
			cudaStreamSynchronize(xs);
			cudaStreamDestroy(xs);
		}
	if (xe_main) cudaEventDestroy(xe_main);
	for (cudaEvent_t e : xe_conv)
		if (e) cudaEventDestroy(e);
	for (cudaEvent_t e : xe_in)
		if (e) cudaEventDestroy(e);
	for (cudaEvent_t e : xe_d2h)
		if (e) cudaEventDestroy(e);
	x_out.free();
	x_in.free();
	if (io_stream) cudaStreamDestroy(io_stream);
	if (io_ready) cudaEventDestroy(io_ready);
	if (io_host) cudaFreeHost(io_host);
	io_dev.free();
	if (stream) cudaStreamSynchronize(stream);
	for (int k = 0; k < 2; k++) {
		if (graph_exec[k]) cudaGraphExecDestroy(graph_exec[k]);
		if (graph[k]) cudaGraphDestroy(graph[k]);
	}
	if (side) cudaStreamDestroy(side);
	if (ev_fork) cudaEventDestroy(ev_fork);
	if (ev_join) cudaEventDestroy(ev_join);
	work.free();
	DevBuf<double>* d[] = {&m, &h, &qw0, &fcx, &fcy, &X, &Y};
	for (auto* p : d) p->free();
	for (int k = 0; k < 4; k++) {
		for (int q = 0; q < 8; q++) sd[k][q].free();
		for (int q = 0; q < 4; q++) sf[k][q].free();
	}
	body_of.free(); params.free(); geom.free(); bbox.free(); total_cells.free(); keys.free(); keys_sorted.free();
	perm_in.free(); perm.free(); cell_start.free(); rec_body.free(); rec.free(); rec2.free(); sort_tmp.free();
	{
		DevBuf<uint32_t>* w32s[] = {&gp_body, &g_sl, &g_snbr, &t_sl, &t_snbr, &p_sl, &p_snbr};
		for (auto* p : w32s) p->free();
		g_cnt.free(); t_cnt.free(); p_cnt.free();
		gp_x.free(); gp_y.free(); gp_qw.free(); gp_hh.free(); gp_ux.free(); gp_uy.free(); gP64.free(); gP32.free(); wpack.free();
		for (int k = 0; k < 3; k++)
			for (int q = 0; q < 4; q++) { gsd[k][q].free(); gsf[k][q].free(); }
		g_w64.free(); t_w64.free(); p_w64.free(); g_w32.free(); t_w32.free(); p_w32.free();
	}
	sl_off.free(); snbr.free(); scnt.free(); sw64.free(); sw32.free(); swA32.free(); recA.free(); recB.free(); dA32.free();
	recB2.free(); sW64.free(); R64.free(); av64.free();
	cm_sw.free(); cm_swA.free(); cm_sX.free(); cm_swji.free(); cm_sW.free();
	cm_U.free(); cm_X.free(); cm_V.free(); cm_P.free(); cm_R.free(); cm_H.free();
	{
		DevBuf<uint32_t>* uws[] = {&uw_gbody, &uw_pc_off, &uw_pc_nbr, &uw_gc_off, &uw_gc_nbr, &uw_pc_cnt, &uw_gc_cnt,
		                           &uw_tp_off, &uw_tp_cnt, &uw_tp_gp,
		                           &uw_tp_slot, &uw_bc_of, &uw_quads};
		for (auto* p : uws) p->free();
		uw_pmask.free(); uw_gmask.free(); uw_ff.free(); uw_vol.free(); uw_vff.free(); uw_qw32.free(); uw_qwlo.free();
		uw_gsig32.free();
		DevBuf<double>* uwd[] = {&uw_pw, &uw_pwx, &uw_pwy, &uw_gw, &uw_gwx, &uw_gwy, &uw_gsig, &uw_ph, &uw_gh, &uw_qwp,
		                         &uw_qws, &uw_gm, &uw_gqw};
		for (auto* p : uwd) p->free();
		for (int k = 0; k < 4; k++)
			for (int q = 0; q < 6; q++) uw_g[k][q].free();
	}
	tt_rows.free(); tt_halo_off.free(); tt_halo.free(); tt_sl.free(); tt_cnt.free(); tt_loc.free(); tt_sw.free();
	tt_swA.free();
	rw_sl.free(); rw_runs.free(); rw_cnt.free(); rw_XF.free(); rw_G.free();
	failed.free();
	DevBuf<uint32_t>* u32s[] = {&nbr_off, &nbr, &bc_rows, &bnd_rows, &bnd_start, &bnd_len, &tile_first, &tile_end,
	                            &slave_rows, &slave_master, &m_tile_off, &m_tile_n};
	for (auto* p : u32s) p->free();
	DevBuf<double>* f64s[] = {&wx64, &wy64, &P64, &dA64, &c64, &bc_v, &slave_dt};
	for (auto* p : f64s) p->free();
	DevBuf<float>* f32s[] = {&qw32, &m32, &h32};
	for (auto* p : f32s) p->free();
	bnd.free(); bnd_ff.free(); tile_bb.free(); staging.free(); mon.free(); mon_counter.free();
	for (auto e : timing.pool) cudaEventDestroy(e);
	if (d_status) cudaFree(d_status);
	if (h_status) cudaFreeHost(h_status);
	if (stream) cudaStreamDestroy(stream);
}

// ================================================================== C ABI
extern "C" {

MF_API const char* mf_status_string(mf_status s) {
	switch (s) {
	case MF_OK: return "ok";
	case MF_ERR_ARG: return "invalid argument";
	case MF_ERR_CUDA: return "CUDA error";
	case MF_ERR_NBH_OVERFLOW: return "neighbour capacity reached";
	case MF_ERR_NONFINITE: return "non-finite state";
	case MF_ERR_TIMEOUT: return "device wait timed out";
	case MF_ERR_PIPELINE: return "unsupported action list";
	case MF_ERR_GRID: return "invalid cell grid";
	case MF_ERR_STATE: return "invalid call for the context state";
	case MF_ERR_NO_DEVICE: return "no CUDA device";
	case MF_ERR_SINGULAR: return "singular corrector matrix";
	case MF_ERR_NO_NEIGHBOR: return "particle without neighbours";
	case MF_ERR_CAPACITY: return "size beyond the documented maximum";
	case MF_ERR_BODY_FAILED: return "some bodies failed (masked; the others stepped on)";
	}
	return "unknown status";
}

MF_API const char* mf_last_error(const mf_ctx* c) { return c ? c->err.c_str() : "null context"; }

MF_API mf_status mf_create(const mf_config* cfg, mf_ctx** out) {
	if (!cfg || !out) return MF_ERR_ARG;
	*out = nullptr;
	if (cfg->method < MF_METHOD_UL || cfg->method > MF_METHOD_UL_WEAK) return MF_ERR_ARG;
	if (cfg->precision < MF_PREC_FP64_STRICT || cfg->precision > MF_PREC_MIXED) return MF_ERR_ARG;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MF_ERR_NO_DEVICE;
	if (cfg->device < 0 || cfg->device >= ndev) return MF_ERR_ARG;
	if (cudaSetDevice(cfg->device) != cudaSuccess) return MF_ERR_CUDA;
	mf_ctx* c = new mf_ctx();
	c->cfg = *cfg;
	cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, cfg->device);
	if (c->cfg.max_nbh == 0) c->cfg.max_nbh = REF_MAX_NBH;
	if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaMalloc(&c->d_status, sizeof(DevStatusH)) != cudaSuccess ||
	    cudaMallocHost(&c->h_status, sizeof(DevStatusH)) != cudaSuccess) {
		delete c;
		return MF_ERR_CUDA;
	}
	c->h_status->flags = 0;
	c->h_status->first_index = 0xffffffffu;
	cudaMemcpy(c->d_status, c->h_status, sizeof(DevStatusH), cudaMemcpyHostToDevice);
	*out = c;
	return MF_OK;
}

MF_API void mf_destroy(mf_ctx* c) { delete c; }

MF_API mf_status mf_add_body(mf_ctx* c, const mf_particles* p, uint32_t n, const mf_sim_data* sd, double dt,
                             int32_t group, int32_t* body_id) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "bodies must be added before the first step");
	if (!p || !sd || n == 0) return fail(c, MF_ERR_ARG, "null particles/sim_data or n == 0");
	if (!(dt > 0.)) return fail(c, MF_ERR_ARG, "dt must be positive");
	if ((uint64_t)c->n_total + n >= 0x7fffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^31 particles");
	const double* src[13] = {p->x, p->y, p->X, p->Y, p->m, p->rho, p->h, p->quad_weight, p->vx, p->vy, p->Sxx, p->Sxy, p->Syy};
	for (int k = 0; k < 13; k++)
		if (!src[k] && k != 2 && k != 3) return fail(c, MF_ERR_ARG, "particle field %d is null", k);
	HostBody b;
	b.off = c->n_total;
	b.n = n;
	b.sd = *sd;
	b.dt = dt;
	b.group = group;
	for (int k = 0; k < 13; k++) {
		const double* s = src[k] ? src[k] : (k == 2 ? p->x : p->y);
		b.in[k].assign(s, s + n);
	}
	c->n_total += n;
	c->bodies.push_back(std::move(b));
	if (body_id) *body_id = (int32_t)c->bodies.size() - 1;
	return MF_OK;
}

MF_API mf_status mf_add_action(mf_ctx* c, int32_t body, int32_t action) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "actions must be added before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	if (action < 1 || action > MF_CONTMECH_ADVECTION_GP) return fail(c, MF_ERR_ARG, "bad action id %d", action);
	c->bodies[body].actions.push_back(action);
	return MF_OK;
}

MF_API mf_status mf_add_boundary_condition(mf_ctx* c, int32_t body, const uint32_t* idx, uint32_t k, int32_t kind,
                                           double value) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "boundary conditions must be added before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	if (kind != MF_BC_PULL && kind != MF_BC_VELOCITY)
		return fail(c, MF_ERR_ARG, "unknown boundary-condition kind %d", kind);
	if (k && !idx) return fail(c, MF_ERR_ARG, "null index list");
	for (uint32_t i = 0; i < k; i++)
		if (idx[i] >= c->bodies[body].n) return fail(c, MF_ERR_ARG, "boundary index %u out of range", idx[i]);
	c->bodies[body].bcs.push_back(HostBC{kind, value, std::vector<uint32_t>(idx, idx + k)});
	return MF_OK;
}

MF_API mf_status mf_set_boundary(mf_ctx* c, int32_t body, const uint32_t* idx, uint32_t nb) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "boundaries must be set before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	if (nb && !idx) return fail(c, MF_ERR_ARG, "null index list");
	for (uint32_t i = 0; i < nb; i++)
		if (idx[i] >= c->bodies[body].n) return fail(c, MF_ERR_ARG, "boundary index %u out of range", idx[i]);
	c->bodies[body].hull.assign(idx, idx + nb);
	return MF_OK;
}

MF_API mf_status mf_set_gauss_mesh(mf_ctx* c, int32_t body, uint32_t ex, uint32_t ey, double gp_h, double gp_rho) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "the mesh must be set before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	HostBody& b = c->bodies[body];
	if (ex == 0 || ey == 0 || (uint64_t)(ex + 1) * (ey + 1) != b.n)
		return fail(c, MF_ERR_ARG, "(ex+1)*(ey+1) must equal the body's particle count");
	if (!(gp_h > 0.) || !(gp_rho > 0.)) return fail(c, MF_ERR_ARG, "Gauss-point h and rho must be positive");
	b.ex = ex; b.ey = ey; b.gp_h = gp_h; b.gp_rho = gp_rho;
	b.quads.clear(); b.order = 2; b.shape = MF_SHAPE_RKPM;
	return MF_OK;
}

MF_API mf_status mf_set_elements(mf_ctx* c, int32_t body, const uint32_t* quads, uint32_t n_elem, uint32_t order,
                                 int32_t shape, double gp_h, double gp_rho) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "the elements must be set before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	HostBody& b = c->bodies[body];
	if (!quads || n_elem == 0) return fail(c, MF_ERR_ARG, "null element map or n_elem == 0");
	if (order != 1 && order != 2) return fail(c, MF_ERR_ARG, "Gauss orders 1 and 2 only");
	if (shape != MF_SHAPE_RKPM && shape != MF_SHAPE_ELEMENT) return fail(c, MF_ERR_ARG, "bad shape kind %d", shape);
	if (c->cfg.method != MF_METHOD_TL_WEAK && c->cfg.method != MF_METHOD_UL_WEAK)
		return fail(c, MF_ERR_ARG, "element maps belong to the weak forms");
	if (c->cfg.method == MF_METHOD_UL_WEAK && shape != MF_SHAPE_ELEMENT)
		return fail(c, MF_ERR_ARG, "a UL_WEAK element map takes MF_SHAPE_ELEMENT (RKPM there is the ellipse's)");
	if ((uint64_t)n_elem * order * order > 0x7fffffffull) return fail(c, MF_ERR_CAPACITY, "more than 2^31 Gauss points");
	for (uint64_t k = 0; k < 4ull * n_elem; k++)
		if (quads[k] >= b.n) return fail(c, MF_ERR_ARG, "element %llu names particle %u of %u", (unsigned long long)(k / 4), quads[k], b.n);
	b.quads.assign(quads, quads + 4ull * n_elem);
	b.ex = b.ey = 0;
	b.order = order; b.shape = shape; b.gp_h = gp_h; b.gp_rho = gp_rho;
	return MF_OK;
}

MF_API mf_status mf_set_gauss_points(mf_ctx* c, int32_t body, const double* x, const double* y, const double* h,
                                     const double* rho, uint32_t n) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "Gauss points must be set before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	if (!x || !y || !h || !rho || n == 0) return fail(c, MF_ERR_ARG, "null Gauss-point field or n == 0");
	HostBody& b = c->bodies[body];
	const double* src[4] = {x, y, h, rho};
	for (int k = 0; k < 4; k++) b.gpt[k].assign(src[k], src[k] + n);
	return MF_OK;
}

MF_API mf_status mf_set_stress_points(mf_ctx* c, int32_t body, const mf_particles* sp, uint32_t n) {
	if (!c) return MF_ERR_ARG;
	if (c->ready) return fail(c, MF_ERR_STATE, "stress points must be set before the first step");
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	if (!sp || n == 0) return fail(c, MF_ERR_ARG, "null stress points or n == 0");
	const double* src[13] = {sp->x, sp->y, sp->X, sp->Y, sp->m, sp->rho, sp->h, sp->quad_weight, sp->vx, sp->vy,
	                         sp->Sxx, sp->Sxy, sp->Syy};
	for (int k = 0; k < 13; k++)
		if (!src[k] && k != 2 && k != 3) return fail(c, MF_ERR_ARG, "stress-point field %d is null", k);
	HostBody& b = c->bodies[body];
	b.n_sp = n;
	for (int k = 0; k < 13; k++) {
		const double* s = src[k] ? src[k] : (k == 2 ? sp->x : sp->y);
		b.sp[k].assign(s, s + n);
	}
	return MF_OK;
}

MF_API mf_status mf_convex_hull(const double* x, const double* y, uint32_t n, uint32_t* out_idx, uint32_t* out_n) {
	if ((!x || !y || !out_idx || !out_n) && n) return MF_ERR_ARG;
	if (out_n) *out_n = 0;
	if (n < 3) return MF_ERR_ARG;
	struct P {
		double x, y;
		uint32_t i;
	};
	std::vector<P> pts(n);
	for (uint32_t i = 0; i < n; i++) pts[i] = P{x[i], y[i], i};
	// lexicographic (x, y) order, as leftlower (convex_hull.h:44-58)
	std::sort(pts.begin(), pts.end(), [](const P a, const P b) {
		if (a.x < b.x) return true;
		if (a.x > b.x) return false;
		return a.y < b.y;
	});
	auto ccw = [](const P& a, const P& b, const P& q) { return (b.x - a.x) * (q.y - a.y) - (b.y - a.y) * (q.x - a.x); };
	std::vector<P> hull(n);
	int k = 0;
	for (int i = 0; i < (int)n; ++i) {
		while (k >= 2 && ccw(hull[k - 2], hull[k - 1], pts[i]) < 0) --k;
		hull[k++] = pts[i];
	}
	for (int i = (int)n - 2, t = k + 1; i >= 0; --i) {
		while (k >= t && ccw(hull[k - 2], hull[k - 1], pts[i]) < 0) --k;
		hull[k++] = pts[i];
	}
	for (int i = 0; i < k - 1; i++) out_idx[i] = hull[i].i;
	*out_n = (uint32_t)(k - 1);
	return MF_OK;
}

}  // extern "C"

namespace {

// The launches of one step of every body, in the driver's order (mfree_iwf.cpp:84-97):
// the RK4 step, then the boundary refresh and contact.
mf_status one_step(mf_ctx* c) {
	const bool tl_lists =
	    c->cfg.method == MF_METHOD_TL || c->cfg.method == MF_METHOD_COROT || c->cfg.method == MF_METHOD_POTENTIAL;
	const bool deferred = contact_deferred(c);
	mf_status st = deferred ? MF_OK : contact_flush(c);
	if (st != MF_OK) return st;
	st = c->cfg.method == MF_METHOD_UL        ? ul_step(c)
	     : tl_lists                            ? tl_step_all(c, deferred && c->contact_pending)
	     : c->cfg.method == MF_METHOD_UL_WEAK ? uw_step(c)
	                                           : weak_step(c);
	if (st != MF_OK) return st;
	if (deferred) c->contact_pending = true;  // this step's query runs with the next step
	else if (c->contact_on) st = contact_run(c, c->stream);
	if (st == MF_OK && c->mon_cap) {
		uint32_t nb = (uint32_t)c->bodies.size();
		bool eos = (c->flags & abit(MF_MATERIAL_EOS)) != 0;
		k_monitor<<<nb, 256, 0, c->stream>>>(nb, c->params.p, c->sd[0][2].p, c->sd[0][3].p, c->sd[0][4].p, c->sf[0][0].p,
		                                      c->sd[0][5].p, c->sd[0][6].p, c->sd[0][7].p, c->sf[0][1].p, c->sf[0][2].p,
		                                      c->sf[0][3].p, c->fcx.p, c->fcy.p, eos ? 1u : 0u, c->mon.p,
		                                      c->mon_counter.p, c->mon_cap);
		k_monitor_tick<<<1, 1, 0, c->stream>>>(c->mon_counter.p);
		c->launches += 2;
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess) return cuda_fail(c, e, "monitor");
	}
	return st;
}

void drop_graph(mf_ctx* c) {
	for (int k = 0; k < 2; k++) {
		if (c->graph_exec[k]) cudaGraphExecDestroy(c->graph_exec[k]);
		if (c->graph[k]) cudaGraphDestroy(c->graph[k]);
		c->graph_exec[k] = nullptr;
		c->graph[k] = nullptr;
	}
}

// Capture one step on the context's stream and instantiate it for replay.
// Capture one step on the context's stream and instantiate it for replay; w = 1: the
// step that starts with the pending contact query.
mf_status capture_step(mf_ctx* c, int w) {
	mf_status pst = tl_prepack(c);
	if (pst != MF_OK) return pst;
	const bool pending = c->contact_pending;
	c->contact_pending = w == 1;
	uint64_t l0 = c->launches;
	CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
	mf_status st = one_step(c);
	cudaGraph_t g = nullptr;
	cudaError_t e = cudaStreamEndCapture(c->stream, &g);
	c->contact_pending = pending;
	if (st != MF_OK) {
		if (g) cudaGraphDestroy(g);
		return st;
	}
	if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
	c->graph[w] = g;
	CK(cudaGraphInstantiate(&c->graph_exec[w], g, 0));
	c->graph_launches[w] = c->launches - l0;
	c->launches = l0;
	return MF_OK;
}

}  // namespace

extern "C" {

MF_API mf_status mf_step(mf_ctx* c, int32_t nsteps) {
	if (!c) return MF_ERR_ARG;
	if (nsteps < 0) return fail(c, MF_ERR_ARG, "nsteps < 0");
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	CK(cudaSetDevice(c->cfg.device));
	bool use_graph = c->cfg.graph && !c->timing.on;
	const bool deferred = contact_deferred(c);
	if (use_graph && c->graph_deferred != deferred) drop_graph(c);  // captured for the other contact order
	c->graph_deferred = deferred;
	for (int32_t k = 0; k < nsteps; k++) {
		if (use_graph) {
			if (!deferred && (st = contact_flush(c)) != MF_OK) return st;
			const int w = deferred && c->contact_pending ? 1 : 0;
			if (!c->graph_exec[w] && (st = capture_step(c, w)) != MF_OK) return st;
			CK(cudaGraphLaunch(c->graph_exec[w], c->stream));
			c->launches += c->graph_launches[w];
			if (deferred) c->contact_pending = true;
		} else {
			st = one_step(c);
			if (st != MF_OK) return st;
		}
		for (auto& b : c->bodies) b.time += b.dt;  // rk4.h:107 (each body's own clock)
	}
	if (c->async_steps) return MF_OK;  // mf_synchronize reads the status
	if ((st = check_status(c)) != MF_OK) return st;
	return failed_status(c);
}

MF_API mf_status mf_synchronize(mf_ctx* c) {
	if (!c) return MF_ERR_ARG;
	if (!c->ready) return MF_OK;
	for (cudaStream_t xs : {c->xs_d2h, c->xs_h2d})
		if (xs) CK(cudaStreamSynchronize(xs));
	std::fill(c->xe_pending, c->xe_pending + 10, false);
	mf_status st = check_status(c);
	return st != MF_OK || !c->async_steps ? st : failed_status(c);  // (synchronous steps report failures themselves)
}

MF_API mf_status mf_get_state(mf_ctx* c, int32_t body, const mf_state* out) {
	if (!c || !out) return MF_ERR_ARG;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	mf_status fst = contact_flush(c);
	if (fst != MF_OK) return fst;
	const HostBody& b = c->bodies[body];
	if (!c->ready) {
		double* o[10] = {out->x, out->y, out->vx, out->vy, out->rho, out->Sxx, out->Sxy, out->Syy, out->fcx, out->fcy};
		const int fld[8] = {0, 1, 8, 9, 5, 10, 11, 12};
		for (int q = 0; q < 8; q++)
			if (o[q]) std::copy(b.in[fld[q]].begin(), b.in[fld[q]].end(), o[q]);
		for (int q = 8; q < 10; q++)
			if (o[q]) std::fill(o[q], o[q] + b.n, 0.);
		return MF_OK;
	}
	CK(cudaSetDevice(c->cfg.device));
	double* o[8] = {out->x, out->y, out->vx, out->vy, out->rho, out->Sxx, out->Sxy, out->Syy};
	if (c->mixed && !c->staging.p) CK(c->staging.alloc(4 * (size_t)c->n_total));
	for (int q = 0; q < 8; q++) {
		if (!o[q]) continue;
		if (c->mixed && q >= 4) {
			double* st = c->staging.p + (size_t)(q - 4) * c->n_total;
			k_f32_to_f64<<<(b.n + 255) / 256, 256, 0, c->stream>>>(b.n, c->sf[0][q - 4].p + b.off, st,
			                                                     q == 4 ? b.sd.rho0 : 0.);
			CK(cudaMemcpyAsync(o[q], st, b.n * 8, cudaMemcpyDeviceToHost, c->stream));
		} else {
			CK(cudaMemcpyAsync(o[q], c->sd[0][q].p + b.off, b.n * 8, cudaMemcpyDeviceToHost, c->stream));
		}
	}
	if (out->fcx) CK(cudaMemcpyAsync(out->fcx, c->fcx.p + b.off, b.n * 8, cudaMemcpyDeviceToHost, c->stream));
	if (out->fcy) CK(cudaMemcpyAsync(out->fcy, c->fcy.p + b.off, b.n * 8, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

MF_API mf_status mf_set_state(mf_ctx* c, int32_t body, const mf_particles* p) {
	if (!c || !p) return MF_ERR_ARG;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	mf_status fst = contact_flush(c);  // the pending query belongs to the positions being replaced
	if (fst != MF_OK) return fst;
	HostBody& b = c->bodies[body];
	const double* src[8] = {p->x, p->y, p->vx, p->vy, p->rho, p->Sxx, p->Sxy, p->Syy};
	const int fld[8] = {0, 1, 8, 9, 5, 10, 11, 12};
	if (!c->ready) {
		for (int q = 0; q < 8; q++)
			if (src[q]) b.in[fld[q]].assign(src[q], src[q] + b.n);
		return MF_OK;
	}
	CK(cudaSetDevice(c->cfg.device));
	if (c->mixed && !c->staging.p) CK(c->staging.alloc(4 * (size_t)c->n_total));
	// TL stage 0 starts from its own copy of the particles (set 2), kept in step
	bool tl = c->cfg.method != MF_METHOD_UL;
	for (int q = 0; q < 8; q++) {
		if (!src[q]) continue;
		if (c->mixed && q >= 4) {
			double* st = c->staging.p + (size_t)(q - 4) * c->n_total;
			CK(cudaMemcpyAsync(st, src[q], b.n * 8, cudaMemcpyHostToDevice, c->stream));
			double off = q == 4 ? b.sd.rho0 : 0.;
			k_f64_to_f32<<<(b.n + 255) / 256, 256, 0, c->stream>>>(b.n, st, c->sf[0][q - 4].p + b.off, off);
			if (tl) k_f64_to_f32<<<(b.n + 255) / 256, 256, 0, c->stream>>>(b.n, st, c->sf[2][q - 4].p + b.off, off);
		} else {
			CK(cudaMemcpyAsync(c->sd[0][q].p + b.off, src[q], b.n * 8, cudaMemcpyHostToDevice, c->stream));
			if (tl) CK(cudaMemcpyAsync(c->sd[2][q].p + b.off, c->sd[0][q].p + b.off, b.n * 8, cudaMemcpyDeviceToDevice, c->stream));
		}
	}
	CK(cudaGetLastError());
	c->tl_recs_valid = false;  // mixed TL: re-pack the records from the new state
	mf_status pst = tl_prepack(c);
	if (pst != MF_OK) return pst;
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

// The device address of host memory the GPU can read and write directly, or null:
// pinned (registered) memory through its mapping, other system memory when the device
// reaches pageable memory through the host's page tables.
const void* device_view(mf_ctx* c, const void* h) {
	if (!h) return nullptr;
	cudaPointerAttributes at{};
	if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	if (at.type == cudaMemoryTypeHost) return at.devicePointer;
	if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return h;
	int pageable = 0;
	cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c->cfg.device);
	return pageable ? h : nullptr;
}

// The fused transfer's device view of the state (set 2 for TL stage 0 when `stage_copy`).
StateIO state_io(mf_ctx* c, bool stage_copy) {
	StateIO io{};
	for (int q = 0; q < 8; q++) {
		const bool f32 = c->mixed && q >= 4;
		io.sd0[q] = f32 ? nullptr : c->sd[0][q].p;
		io.sd2[q] = (f32 || !stage_copy) ? nullptr : c->sd[2][q].p;
		if (f32) {
			io.sf0[q - 4] = c->sf[0][q - 4].p;
			io.sf2[q - 4] = stage_copy ? c->sf[2][q - 4].p : nullptr;
		}
	}
	io.fcx = c->fcx.p;
	io.fcy = c->fcy.p;
	return io;
}

MF_API mf_status mf_get_state_all(mf_ctx* c, const mf_state* out) {
	if (!c || !out) return MF_ERR_ARG;
	mf_status fst = contact_flush(c);
	if (fst != MF_OK) return fst;
	if (!c->ready) {
		for (int32_t b = 0; b < (int32_t)c->bodies.size(); b++) {
			const uint32_t o = c->bodies[b].off;
			auto at = [o](double* p) { return p ? p + o : nullptr; };
			mf_state ob = {at(out->x), at(out->y), at(out->vx), at(out->vy), at(out->rho),
			               at(out->Sxx), at(out->Sxy), at(out->Syy), at(out->fcx), at(out->fcy)};
			mf_status st = mf_get_state(c, b, &ob);
			if (st != MF_OK) return st;
		}
		return MF_OK;
	}
	CK(cudaSetDevice(c->cfg.device));
	const uint32_t n = c->n_total;
	double* o[8] = {out->x, out->y, out->vx, out->vy, out->rho, out->Sxx, out->Sxy, out->Syy};
	{
		StateIO io = state_io(c, false);
		double* all[10] = {o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], out->fcx, out->fcy};
		bool direct = c->cfg.method != MF_METHOD_TL_WEAK && c->cfg.method != MF_METHOD_UL_WEAK;
		for (int q = 0; q < 10 && direct; q++) {
			if (!all[q]) continue;
			io.dst[q] = (double*)device_view(c, all[q]);
			direct = io.dst[q] != nullptr;
		}
		if (direct) {
			if (n) k_get_state_io<<<(n + 255) / 256, 256, 0, c->stream>>>(n, io, c->body_of.p, c->params.p);
			CK(cudaGetLastError());
			CK(cudaStreamSynchronize(c->stream));
			return MF_OK;
		}
	}
	if (c->mixed && !c->staging.p) CK(c->staging.alloc(4 * (size_t)n));
	for (int q = 0; q < 8; q++) {
		if (!o[q]) continue;
		if (c->mixed && q >= 4) {
			double* st = c->staging.p + (size_t)(q - 4) * n;
			k_f32_to_f64_rows<<<(n + 255) / 256, 256, 0, c->stream>>>(n, c->sf[0][q - 4].p, st, c->body_of.p, c->params.p,
			                                                        q == 4);
			CK(cudaMemcpyAsync(o[q], st, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
		} else {
			CK(cudaMemcpyAsync(o[q], c->sd[0][q].p, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
		}
	}
	if (out->fcx) CK(cudaMemcpyAsync(out->fcx, c->fcx.p, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
	if (out->fcy) CK(cudaMemcpyAsync(out->fcy, c->fcy.p, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

MF_API mf_status mf_set_state_all(mf_ctx* c, const mf_particles* p) {
	if (!c || !p) return MF_ERR_ARG;
	mf_status fst = contact_flush(c);
	if (fst != MF_OK) return fst;
	if (!c->ready) {
		for (int32_t b = 0; b < (int32_t)c->bodies.size(); b++) {
			const uint32_t o = c->bodies[b].off;
			auto at = [o](const double* q) { return q ? q + o : nullptr; };
			mf_particles pb = {at(p->x), at(p->y), nullptr, nullptr, nullptr, at(p->rho), nullptr, nullptr,
			                   at(p->vx), at(p->vy), at(p->Sxx), at(p->Sxy), at(p->Syy)};
			mf_status st = mf_set_state(c, b, &pb);
			if (st != MF_OK) return st;
		}
		return MF_OK;
	}
	CK(cudaSetDevice(c->cfg.device));
	const uint32_t n = c->n_total;
	const double* src[8] = {p->x, p->y, p->vx, p->vy, p->rho, p->Sxx, p->Sxy, p->Syy};
	const bool tl = c->cfg.method != MF_METHOD_UL;  // TL stage 0 starts from its own copy (set 2)
	{
		StateIO io = state_io(c, tl);
		bool direct = c->cfg.method != MF_METHOD_TL_WEAK && c->cfg.method != MF_METHOD_UL_WEAK;
		for (int q = 0; q < 8 && direct; q++) {
			if (!src[q]) continue;
			io.src[q] = (const double*)device_view(c, src[q]);
			direct = io.src[q] != nullptr;
		}
		if (direct) {
			if (n) k_set_state_io<<<(n + 255) / 256, 256, 0, c->stream>>>(n, io, c->body_of.p, c->params.p);
			CK(cudaGetLastError());
			c->tl_recs_valid = false;  // mixed TL: re-pack the records from the new state
			mf_status pst = tl_prepack(c);
			if (pst != MF_OK) return pst;
			CK(cudaStreamSynchronize(c->stream));
			return MF_OK;
		}
	}
	if (c->mixed && !c->staging.p) CK(c->staging.alloc(4 * (size_t)n));
	for (int q = 0; q < 8; q++) {
		if (!src[q]) continue;
		if (c->mixed && q >= 4) {
			double* st = c->staging.p + (size_t)(q - 4) * n;
			CK(cudaMemcpyAsync(st, src[q], (size_t)n * 8, cudaMemcpyHostToDevice, c->stream));
			k_f64_to_f32_rows<<<(n + 255) / 256, 256, 0, c->stream>>>(n, st, c->sf[0][q - 4].p, c->body_of.p, c->params.p,
			                                                        q == 4);
			if (tl) CK(cudaMemcpyAsync(c->sf[2][q - 4].p, c->sf[0][q - 4].p, (size_t)n * 4, cudaMemcpyDeviceToDevice, c->stream));
		} else {
			CK(cudaMemcpyAsync(c->sd[0][q].p, src[q], (size_t)n * 8, cudaMemcpyHostToDevice, c->stream));
			if (tl) CK(cudaMemcpyAsync(c->sd[2][q].p, c->sd[0][q].p, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->stream));
		}
	}
	CK(cudaGetLastError());
	c->tl_recs_valid = false;  // mixed TL: re-pack the records from the new state
	mf_status pst = tl_prepack(c);
	if (pst != MF_OK) return pst;
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

// ---- stream-ordered transfers of all bodies' state
namespace {
mf_status xfer_setup(mf_ctx* c) {
	if (c->xs_d2h) return MF_OK;
	CK(cudaStreamCreateWithFlags(&c->xs_d2h, cudaStreamNonBlocking));
	CK(cudaStreamCreateWithFlags(&c->xs_h2d, cudaStreamNonBlocking));
	CK(cudaEventCreateWithFlags(&c->xe_main, cudaEventDisableTiming));
	for (auto& e : c->xe_d2h) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
	for (auto& e : c->xe_conv) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
	for (auto& e : c->xe_in) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
	CK(c->x_out.alloc(10 * (size_t)c->n_total));
	CK(c->x_in.alloc(8 * (size_t)c->n_total));
	return MF_OK;
}
}  // namespace

// The state of every body into out (host memory, pinned for the copies to run
// asynchronously): stream-ordered after the steps already queued; returns at once.
// The fields are valid after mf_synchronize.  One kernel writes all fields as FP64
// into device staging, then each field goes to the host by its own copy on the
// device->host copy stream.
MF_API mf_status mf_get_state_all_async(mf_ctx* c, const mf_state* out) {
	if (!c || !out) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = contact_flush(c)) != MF_OK) return st;
	if (c->cfg.method == MF_METHOD_TL_WEAK || c->cfg.method == MF_METHOD_UL_WEAK)
		return fail(c, MF_ERR_PIPELINE, "the asynchronous transfers cover the strong forms");
	CK(cudaSetDevice(c->cfg.device));
	if ((st = xfer_setup(c)) != MF_OK) return st;
	const uint32_t n = c->n_total;
	double* o[10] = {out->x, out->y, out->vx, out->vy, out->rho, out->Sxx, out->Sxy, out->Syy, out->fcx, out->fcy};
	// field by field: each field's staging is rewritten once the previous get's copy of
	// it has left, converted by its own small kernel, and sent at once -- the copies of
	// the first fields run while the later ones convert
	const StateIO io = state_io(c, false);
	for (int q = 0; q < 10; q++) {
		if (o[q]) {
			StateIO one = io;
			for (int r = 0; r < 10; r++) one.dst[r] = r == q ? c->x_out.p + (size_t)q * n : nullptr;
			CK(cudaStreamWaitEvent(c->stream, c->xe_d2h[q], 0));
			if (n) k_get_state_io<<<(n + 255) / 256, 256, 0, c->stream>>>(n, one, c->body_of.p, c->params.p);
			CK(cudaGetLastError());
			CK(cudaEventRecord(c->xe_conv[q], c->stream));
			CK(cudaStreamWaitEvent(c->xs_d2h, c->xe_conv[q], 0));
			CK(cudaMemcpyAsync(o[q], c->x_out.p + (size_t)q * n, (size_t)n * 8, cudaMemcpyDeviceToHost, c->xs_d2h));
			c->xe_pending[q] = true;
		}
		CK(cudaEventRecord(c->xe_d2h[q], c->xs_d2h));
	}
	return MF_OK;
}

// Overwrite the state of every body from p (host memory, pinned): stream-ordered;
// returns at once, and the host arrays may be reused after mf_synchronize.  Each field
// is copied on the host->device copy stream, after the device->host copy of the same
// field by an earlier mf_get_state_all_async (so a get followed by a set of the same
// host arrays reads what the get wrote, and the two directions overlap field by field);
// then one kernel writes the device state from the staging.
MF_API mf_status mf_set_state_all_async(mf_ctx* c, const mf_particles* p) {
	if (!c || !p) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = contact_flush(c)) != MF_OK) return st;
	if (c->cfg.method == MF_METHOD_TL_WEAK || c->cfg.method == MF_METHOD_UL_WEAK)
		return fail(c, MF_ERR_PIPELINE, "the asynchronous transfers cover the strong forms");
	CK(cudaSetDevice(c->cfg.device));
	if ((st = xfer_setup(c)) != MF_OK) return st;
	const uint32_t n = c->n_total;
	const double* src[8] = {p->x, p->y, p->vx, p->vy, p->rho, p->Sxx, p->Sxy, p->Syy};
	// the staging is rewritten only after the previous set's kernels have read it; then
	// field by field: copied in, and converted into the state by its own small kernel as
	// soon as it has arrived (the later fields' copies run meanwhile)
	CK(cudaEventRecord(c->xe_main, c->stream));
	CK(cudaStreamWaitEvent(c->xs_h2d, c->xe_main, 0));
	const StateIO io = state_io(c, c->cfg.method != MF_METHOD_UL);  // TL stage 0 starts from its own copy (set 2)
	// mixed TL: the stage-0 records packed in parts as their fields land (positions after
	// y, velocities after vy, {h, m, rho, c} after rho), off the path to the step
	const bool parts = c->cfg.method == MF_METHOD_TL && c->mixed && !c->n_bc && src[0] && src[1] && src[2] && src[3] &&
	                   src[4];
	TLArgs ta{};
	if (parts) {
		ta = tl_args(c);
		ta.stage = 0;
		ta.recB = c->recB.p;
	}
	for (int q = 0; q < 8; q++) {
		if (!src[q]) continue;
		if (c->xe_pending[q]) CK(cudaStreamWaitEvent(c->xs_h2d, c->xe_d2h[q], 0));
		CK(cudaMemcpyAsync(c->x_in.p + (size_t)q * n, src[q], (size_t)n * 8, cudaMemcpyHostToDevice, c->xs_h2d));
		CK(cudaEventRecord(c->xe_in[q], c->xs_h2d));
		CK(cudaStreamWaitEvent(c->stream, c->xe_in[q], 0));
		StateIO one = io;
		for (int r = 0; r < 8; r++) one.src[r] = r == q ? c->x_in.p + (size_t)q * n : nullptr;
		if (n) k_set_state_io<<<(n + 255) / 256, 256, 0, c->stream>>>(n, one, c->body_of.p, c->params.p);
		CK(cudaGetLastError());
		const int part = q == 1 ? 6 : q == 3 ? 7 : q == 4 ? 8 : 0;
		if (parts && part) {
			cudaError_t e = tl_launch(c, ta, part);
			if (e != cudaSuccess) return cuda_fail(c, e, "tl pack");
			c->launches++;
		}
	}
	if (parts) {
		c->tl_recs_valid = true;
		return MF_OK;
	}
	c->tl_recs_valid = false;  // mixed TL: re-pack the records from the new state
	return tl_prepack(c);
}

// The stress the method evaluates at the body's current state.  TL (strong form):
// pass A once more on the current state -- the displacement gradient, Green-St Venant
// and the nominal stress P = J F^-1 sigma (derivatives.h:101-149, material.h:132-161,
// cont_mech.h:154-169) -- into the per-stage scratch the next step rewrites anyway;
// UL: the state's stress S (P_xy = P_yx = S_xy).
MF_API mf_status mf_get_stress(mf_ctx* c, int32_t body, double* Pxx, double* Pxy, double* Pyx, double* Pyy) {
	if (!c || !Pxx || !Pxy || !Pyx || !Pyy) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = contact_flush(c)) != MF_OK) return st;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "no body %d", body);
	const HostBody& b = c->bodies[body];
	if (c->cfg.method == MF_METHOD_UL) {
		mf_state o{};
		o.Sxx = Pxx; o.Sxy = Pxy; o.Syy = Pyy;
		if ((st = mf_get_state(c, body, &o)) != MF_OK) return st;
		std::copy(Pxy, Pxy + b.n, Pyx);
		return MF_OK;
	}
	if (c->cfg.method != MF_METHOD_TL)
		return fail(c, MF_ERR_STATE, "the stress evaluation covers the UL and the strong-form TL methods");
	CK(cudaSetDevice(c->cfg.device));
	TLArgs a = tl_args(c);
	a.stage = 0;
	a.recB = c->recB.p;  // stage 0 reads set 2 and (mixed) the first record buffer
	cudaError_t e;
	if (c->mixed && (c->n_bc || !c->tl_recs_valid) && (e = tl_launch(c, a, 1)) != cudaSuccess)
		return cuda_fail(c, e, "tl pack");
	if ((e = tl_launch(c, a, 2)) != cudaSuccess) return cuda_fail(c, e, "tl pass A");
	const uint32_t n = b.n, o = b.off;
	double* out[4] = {Pxx, Pxy, Pyx, Pyy};
	if (c->mixed) {  // P is the records' first field array (float4 per row)
		std::vector<float> h(4 * (size_t)n);
		CK(cudaMemcpyAsync(h.data(), c->recB.p + o, 16ull * n, cudaMemcpyDeviceToHost, c->stream));
		CK(cudaStreamSynchronize(c->stream));
		for (uint32_t i = 0; i < n; i++)
			for (int k = 0; k < 4; k++) out[k][i] = h[4 * (size_t)i + k];
	} else {
		for (int k = 0; k < 4; k++)
			CK(cudaMemcpyAsync(out[k], c->P64.p + (size_t)k * c->n_total + o, (size_t)n * 8, cudaMemcpyDeviceToHost,
			                   c->stream));
		CK(cudaStreamSynchronize(c->stream));
	}
	return check_status(c);
}

// The weak TL form's Gauss-point state (rho, Sxx, Sxy, Syy) of every body, the bodies'
// points concatenated in id order.
MF_API mf_status mf_get_gauss_state(mf_ctx* c, double* rho, double* Sxx, double* Sxy, double* Syy, uint32_t cap,
                                    uint32_t* n_out) {
	if (!c || !n_out) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if (c->cfg.method != MF_METHOD_TL_WEAK && c->cfg.method != MF_METHOD_UL_WEAK)
		return fail(c, MF_ERR_STATE, "Gauss points and stress points belong to the weak forms");
	const uint32_t ng = c->n_g;
	*n_out = ng;
	if (!rho && !Sxx && !Sxy && !Syy) return MF_OK;
	if (cap < ng) return fail(c, MF_ERR_ARG, "capacity %u below the %u Gauss points", cap, ng);
	CK(cudaSetDevice(c->cfg.device));
	CK(cudaStreamSynchronize(c->stream));
	double* out[4] = {rho, Sxx, Sxy, Syy};
	if (c->cfg.method == MF_METHOD_UL_WEAK) {  // the stress points' state (FP64 in every form)
		for (int q = 0; q < 4; q++)
			if (out[q]) CK(cudaMemcpy(out[q], c->uw_g[0][2 + q].p, (size_t)ng * 8, cudaMemcpyDeviceToHost));
		return check_status(c);
	}
	if (c->mixed) {
		std::vector<uint32_t> gb(ng);
		CK(cudaMemcpy(gb.data(), c->gp_body.p, (size_t)ng * 4, cudaMemcpyDeviceToHost));
		std::vector<float> h(ng);
		for (int q = 0; q < 4; q++) {
			if (!out[q]) continue;
			CK(cudaMemcpy(h.data(), c->gsf[0][q].p, (size_t)ng * 4, cudaMemcpyDeviceToHost));
			for (uint32_t g = 0; g < ng; g++)  // the mixed form keeps rho - rho0
				out[q][g] = (double)h[g] + (q == 0 ? c->bodies[gb[g]].sd.rho0 : 0.);
		}
	} else {
		for (int q = 0; q < 4; q++)
			if (out[q]) CK(cudaMemcpy(out[q], c->gsd[0][q].p, (size_t)ng * 8, cudaMemcpyDeviceToHost));
	}
	return check_status(c);
}

MF_API mf_status mf_get_failed(mf_ctx* c, uint32_t* flags, uint32_t n_bodies) {
	if (!c || !flags) return MF_ERR_ARG;
	if (n_bodies < c->bodies.size()) return fail(c, MF_ERR_ARG, "room for %u of %zu bodies", n_bodies, c->bodies.size());
	if (!c->ready) {
		std::fill(flags, flags + c->bodies.size(), 0u);
		return MF_OK;
	}
	CK(cudaStreamSynchronize(c->stream));
	CK(cudaMemcpy(flags, c->failed.p, c->bodies.size() * 4, cudaMemcpyDeviceToHost));
	return MF_OK;
}

MF_API mf_status mf_get_time(mf_ctx* c, int32_t body, double* t) {
	if (!c || !t) return MF_ERR_ARG;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	*t = c->bodies[body].time;
	return MF_OK;
}

MF_API mf_status mf_num_particles(mf_ctx* c, int32_t body, uint32_t* n) {
	if (!c || !n) return MF_ERR_ARG;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	*n = c->bodies[body].n;
	return MF_OK;
}

MF_API mf_status mf_get_neighbors(mf_ctx* c, int32_t body, uint32_t* counts, uint32_t* idx, uint64_t cap,
                                  uint64_t* total) {
	if (!c || !counts || !total) return MF_ERR_ARG;
	if (body < 0 || body >= (int32_t)c->bodies.size()) return fail(c, MF_ERR_ARG, "bad body id %d", body);
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	const HostBody& b = c->bodies[body];
	uint32_t n = c->n_total;
	std::vector<uint32_t> all_counts(n);
	std::vector<uint64_t> offs(n + 1, 0);
	DevBuf<uint32_t> d_counts, d_idx;
	DevBuf<uint64_t> d_offs;
	CK(d_counts.alloc(n));
	CK(d_offs.alloc(n + 1));
	std::vector<uint32_t> all_idx;
	if (c->cfg.method == MF_METHOD_UL) {
		if (c->mixed) return fail(c, MF_ERR_STATE, "UL neighbour lists are available in the FP64 forms");
		ULArgs a = ul_args(c, 0);
		cudaError_t e = mf_strict::ul_neighbors(a, d_counts.p, nullptr, nullptr, 0, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "ul_neighbors");
		CK(cudaMemcpyAsync(all_counts.data(), d_counts.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
		CK(cudaStreamSynchronize(c->stream));
		for (uint32_t i = 0; i < n; i++) offs[i + 1] = offs[i] + all_counts[i];
		CK(d_idx.alloc(offs[n]));
		CK(cudaMemcpy(d_offs.p, offs.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
		e = mf_strict::ul_neighbors(a, d_counts.p, d_idx.p, d_offs.p, 1, c->stream);
		if (e != cudaSuccess) return cuda_fail(c, e, "ul_neighbors");
		all_idx.resize(offs[n]);
		CK(cudaMemcpyAsync(all_idx.data(), d_idx.p, offs[n] * 4, cudaMemcpyDeviceToHost, c->stream));
		st = check_status(c);
		if (st != MF_OK && st != MF_ERR_NBH_OVERFLOW) return st;
	} else if (c->cfg.method == MF_METHOD_UL_WEAK) {
		// the ellipse neighbourhoods of the particles' current state: those of the next
		// step's first derivative evaluation (on element maps the particles have none)
		if (!c->uw_order) {
			UWArgs a = uw_args(c, 0);
			cudaError_t e = uw_neighbourhoods(c, a, false, false);
			if (e != cudaSuccess) return cuda_fail(c, e, "weak UL neighbourhoods");
		}
		CK(cudaStreamSynchronize(c->stream));
		uint64_t ec = c->uw_pc_nbr.n;
		std::vector<uint32_t> start(n + 1), cnt(n + 1), cand(ec);
		std::vector<uint8_t> mask(ec);
		CK(cudaMemcpy(start.data(), c->uw_pc_off.p, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(cnt.data(), c->uw_pc_cnt.p, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
		if (ec) {
			CK(cudaMemcpy(cand.data(), c->uw_pc_nbr.p, ec * 4, cudaMemcpyDeviceToHost));
			CK(cudaMemcpy(mask.data(), c->uw_pmask.p, ec, cudaMemcpyDeviceToHost));
		}
		st = check_status(c);
		if (st != MF_OK) return st;
		for (uint32_t i = 0; i < n; i++) {
			for (uint64_t k = 0, q = start[i]; k < cnt[i]; k++, q += c->uw_pc_stride)
				if (mask[q]) all_idx.push_back(cand[q]);
			all_counts[i] = (uint32_t)(all_idx.size() - offs[i]);
			offs[i + 1] = all_idx.size();
		}
	} else {
		std::vector<uint32_t> off(n + 1);
		CK(cudaMemcpy(off.data(), c->nbr_off.p, (n + 1) * 4, cudaMemcpyDeviceToHost));
		all_idx.resize(off[n]);
		if (off[n]) CK(cudaMemcpy(all_idx.data(), c->nbr.p, (size_t)off[n] * 4, cudaMemcpyDeviceToHost));
		for (uint32_t i = 0; i < n; i++) { all_counts[i] = off[i + 1] - off[i]; offs[i + 1] = off[i + 1]; }
	}
	d_counts.free(); d_idx.free(); d_offs.free();
	uint64_t tot = 0;
	for (uint32_t i = 0; i < b.n; i++) {
		uint32_t r = b.off + i;
		counts[i] = all_counts[r];
		for (uint64_t q = offs[r]; q < offs[r + 1]; q++) {
			if (idx && tot < cap) idx[tot] = all_idx[q] - b.off;
			tot++;
		}
	}
	*total = tot;
	return MF_OK;
}

MF_API mf_status mf_set_timing(mf_ctx* c, int32_t enable) {
	if (!c) return MF_ERR_ARG;
	c->timing.on = enable != 0;
	for (int k = 0; k < 8; k++) { c->timing.ms[k] = 0.; c->timing.launches[k] = 0; c->timing.rows[k] = 0; }
	return MF_OK;
}

MF_API mf_status mf_kernel_stats(mf_ctx* c, int32_t kind, double* total_ms, uint64_t* launches, uint64_t* rows) {
	if (!c || kind < 0 || kind >= 8) return MF_ERR_ARG;
	if (total_ms) *total_ms = c->timing.ms[kind];
	if (launches) *launches = c->timing.launches[kind];
	if (rows) *rows = c->timing.rows[kind];
	return MF_OK;
}

MF_API mf_status mf_launch_count(mf_ctx* c, uint64_t* launches) {
	if (!c || !launches) return MF_ERR_ARG;
	*launches = c->launches;
	return MF_OK;
}

}  // extern "C"

namespace {

// Device snapshot of everything a step changes (state, contact forces, TL stage-0
// copy, body clocks), so trial steps leave no trace.
struct Snapshot {
	std::vector<DevBuf<unsigned char>> bufs;
	std::vector<std::pair<void*, size_t>> src;
	std::vector<double> times;
	std::vector<BodyParams> params;
};

mf_status snapshot_take(mf_ctx* c, Snapshot& s) {
	uint32_t n = c->n_total;
	auto add = [&](void* p, size_t bytes) -> mf_status {
		if (!p || !bytes) return MF_OK;
		s.bufs.emplace_back();
		CK(s.bufs.back().alloc(bytes));
		CK(cudaMemcpyAsync(s.bufs.back().p, p, bytes, cudaMemcpyDeviceToDevice, c->stream));
		s.src.push_back({p, bytes});
		return MF_OK;
	};
	mf_status st;
	for (int k : {0, 2})
		for (int q = 0; q < 8; q++)
			if ((st = add(c->sd[k][q].p, (size_t)n * 8)) || (k == 0 && q < 4 && (st = add(c->sf[k][q].p, (size_t)n * 4))) ||
			    (k == 2 && q < 4 && (st = add(c->sf[k][q].p, (size_t)n * 4))))
				return st;
	if ((st = add(c->fcx.p, (size_t)n * 8)) || (st = add(c->fcy.p, (size_t)n * 8))) return st;
	if ((st = add(c->params.p, c->h_params.size() * sizeof(BodyParams)))) return st;
	if ((st = add(c->failed.p, c->bodies.size() * 4))) return st;  // trial steps may fail a body
	for (auto& b : c->bodies) s.times.push_back(b.time);
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

mf_status snapshot_restore(mf_ctx* c, Snapshot& s) {
	for (size_t i = 0; i < s.bufs.size(); i++)
		CK(cudaMemcpyAsync(s.src[i].first, s.bufs[i].p, s.src[i].second, cudaMemcpyDeviceToDevice, c->stream));
	c->tl_recs_valid = false;  // mixed TL: re-pack the records from the restored state
	c->contact_pending = false;  // the snapshot holds the forces of its positions
	mf_status pst = tl_prepack(c);
	if (pst != MF_OK) return pst;
	for (size_t b = 0; b < c->bodies.size(); b++) c->bodies[b].time = s.times[b];
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

void snapshot_free(Snapshot& s) {
	for (auto& b : s.bufs) b.free();
}

std::string tune_key(mf_ctx* c) {
	// (method, precision, particle-count bucket, smoothing-length bucket): the launch
	// shapes that win depend on the rows per launch and on the neighbours per row,
	// which the lattice spacing (through h) and the body sizes set
	int bucket = 0;
	while ((1u << bucket) < c->n_total) bucket++;
	double hsum = 0.;
	uint64_t hn = 0;
	for (auto& b : c->bodies)
		for (double h : b.in[6]) {
			hsum += h;
			hn++;
		}
	int hb = hn ? (int)std::floor(std::log2(std::max(hsum / (double)hn, 1e-12))) : 0;
	char k[128];
	// (the mixed TL form also by its pass family: the run walk or the streamed lists)
	snprintf(k, sizeof k, "m%d p%d n2^%d h2^%d r%u", c->cfg.method, c->cfg.precision, bucket, hb, c->tune.tl_runs);
	return k;
}

}  // namespace

extern "C" {

MF_API mf_status mf_autotune(mf_ctx* c, int32_t trial_steps, char* report, uint32_t report_len) {
	if (!c || trial_steps < 1) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = contact_flush(c)) != MF_OK) return st;
	if (c->cfg.method == MF_METHOD_UL_WEAK) {  // fixed launch shapes: nothing to try
		if (report && report_len) snprintf(report, report_len, "fixed launch shapes");
		return MF_OK;
	}
	CK(cudaSetDevice(c->cfg.device));
	std::string key = tune_key(c);
	std::string rep;
	{
		std::lock_guard<std::mutex> lock(g_tune_mutex);
		auto it = g_tune_cache.find(key);
		if (it != g_tune_cache.end()) {
			c->tune = it->second;
			drop_graph(c);
			rep = "cached " + key;
			if (report && report_len) snprintf(report, report_len, "%s", rep.c_str());
			return MF_OK;
		}
	}
	std::vector<Tune> cands;
	for (uint32_t bs : {64u, 128u, 256u}) {
		Tune t = c->tune;
		if (c->cfg.method == MF_METHOD_UL) {
			t.ul_block = bs;
			t.ul_persistent = 0;
			t.ul_chunk = 1;
			t.ul_split = 1;
			cands.push_back(t);
			if (c->mixed)
				for (uint32_t sp : {4u, 8u}) {
					t.ul_split = sp;
					cands.push_back(t);
				}
			t.ul_split = 1;
			for (uint32_t ch : {1u, 4u}) {
				t.ul_persistent = 1;
				t.ul_chunk = ch;
				cands.push_back(t);
			}
		} else {
			t.tl_block = bs;
			t.tl_tiled = 0;
			// (tl_runs stays as set: it changes results in the last FP32 bits; the
			// unroll factor of the run walk does not)
			for (uint32_t u : {1u, 2u, 3u, 4u}) {
				t.tl_unroll = u;
				if (u == 1 || (c->cfg.method == MF_METHOD_TL && c->mixed && c->rw_ok && t.tl_runs)) cands.push_back(t);
			}
		}
	}
	if (c->cfg.method == MF_METHOD_TL && c->mixed && c->tt_ok) {
		Tune t = c->tune;
		t.tl_tiled = 1;  // the tiled passes have a fixed block (one tile)
		cands.push_back(t);
	}
	Snapshot snap;
	if ((st = snapshot_take(c, snap)) != MF_OK) return st;
	bool timing_was = c->timing.on;
	c->timing.on = false;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	double best = 1e300;
	Tune best_t = c->tune;
	char line[160];
	for (const Tune& t : cands) {
		c->tune = t;
		if ((st = snapshot_restore(c, snap)) != MF_OK) break;
		if ((st = one_step(c)) != MF_OK) break;  // warm-up
		cudaEventRecord(e0, c->stream);
		for (int32_t k = 0; k < trial_steps && st == MF_OK; k++) st = one_step(c);
		cudaEventRecord(e1, c->stream);
		if (st != MF_OK) break;
		if ((st = check_status(c)) != MF_OK) break;
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		double per = ms / trial_steps;
		snprintf(line, sizeof line, "%s[b%u p%u c%u s%u tl%u t%u r%u u%u]=%.4fms", rep.empty() ? "" : " ", t.ul_block,
		         t.ul_persistent, t.ul_chunk, t.ul_split, t.tl_block, t.tl_tiled, t.tl_runs, t.tl_unroll, per);
		rep += line;
		if (per < best) {
			best = per;
			best_t = t;
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	c->timing.on = timing_was;
	c->tune = best_t;
	mf_status rs = snapshot_restore(c, snap);
	snapshot_free(snap);
	if (st != MF_OK) return st;
	if (rs != MF_OK) return rs;
	drop_graph(c);
	{
		std::lock_guard<std::mutex> lock(g_tune_mutex);
		g_tune_cache[key] = best_t;
	}
	snprintf(line, sizeof line, " -> b%u p%u c%u s%u tl%u t%u r%u u%u (%s)", best_t.ul_block, best_t.ul_persistent,
	         best_t.ul_chunk, best_t.ul_split, best_t.tl_block, best_t.tl_tiled, best_t.tl_runs, best_t.tl_unroll,
	         key.c_str());
	rep += line;
	if (report && report_len) snprintf(report, report_len, "%s", rep.c_str());
	return MF_OK;
}

MF_API mf_status mf_set_option(mf_ctx* c, const char* key, int64_t value) {
	if (!c || !key) return MF_ERR_ARG;
	if (!strcmp(key, "ul_split")) {
		if (value != 1 && value != 4 && value != 8) return fail(c, MF_ERR_ARG, "ul_split must be 1, 4 or 8");
		c->tune.ul_split = (uint32_t)value;
		c->tune.ul_persistent = 0;
		drop_graph(c);
		return MF_OK;
	}
	if (!strcmp(key, "tl_tiles")) {
		if (value != 0 && value != 1) return fail(c, MF_ERR_ARG, "tl_tiles must be 0 or 1");
		if (value == 1 && c->ready && !c->tt_ok)
			return fail(c, MF_ERR_STATE, "tl_tiles: the halo tiles are built at set-up; set the option before the first step");
		c->tune.tl_tiled = (uint32_t)value;
		drop_graph(c);
		return MF_OK;
	}
	if (!strcmp(key, "mask_failed")) {
		if (value != 0 && value != 1) return fail(c, MF_ERR_ARG, "mask_failed must be 0 or 1");
		if (value && c->cfg.method != MF_METHOD_UL)
			return fail(c, MF_ERR_PIPELINE, "per-body failure masking covers the updated-Lagrangian method");
		c->mask_failed = value != 0;
		drop_graph(c);
		return MF_OK;
	}
	if (!strcmp(key, "async_steps")) {
		if (value != 0 && value != 1) return fail(c, MF_ERR_ARG, "async_steps must be 0 or 1");
		c->async_steps = value != 0;
		return MF_OK;
	}
	if (!strcmp(key, "contact_overlap")) {
		if (value != 0 && value != 1) return fail(c, MF_ERR_ARG, "contact_overlap must be 0 or 1");
		mf_status fst = contact_flush(c);
		if (fst != MF_OK) return fst;
		c->contact_overlap = value != 0;
		drop_graph(c);
		return MF_OK;
	}
	if (!strcmp(key, "tl_runs")) {
		if (value != 0 && value != 1) return fail(c, MF_ERR_ARG, "tl_runs must be 0 or 1");
		c->tune.tl_runs = (uint32_t)value;
		drop_graph(c);
		return MF_OK;
	}
	return fail(c, MF_ERR_ARG, "unknown option '%s'", key);
}

MF_API mf_status mf_get_option(mf_ctx* c, const char* key, int64_t* value) {
	if (!c || !key || !value) return MF_ERR_ARG;
	if (!strcmp(key, "tl_tiles")) {
		*value = c->tune.tl_tiled;
		return MF_OK;
	}
	if (!strcmp(key, "ul_split")) {
		*value = c->tune.ul_split;
		return MF_OK;
	}
	if (!strcmp(key, "contact_overlap")) {
		*value = c->contact_overlap ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "async_steps")) {
		*value = c->async_steps ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "weak_gp_entries")) {
		*value = (int64_t)c->g_entries;
		return MF_OK;
	}
	if (!strcmp(key, "weak_particle_entries")) {
		*value = (int64_t)c->t_entries;
		return MF_OK;
	}
	if (!strcmp(key, "weak_gauss_points")) {
		*value = c->n_g;
		return MF_OK;
	}
	if (!strcmp(key, "tl_runs")) {
		*value = c->tune.tl_runs;
		return MF_OK;
	}
	if (!strcmp(key, "mask_failed")) {
		*value = c->mask_failed ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "tl_runs_built")) {
		*value = c->rw_ok ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "tl_run_words")) {  // run words over all rows (the lists as runs)
		*value = (int64_t)c->rw_words;
		return MF_OK;
	}
	if (!strcmp(key, "tl_tiles_built")) {
		*value = c->tt_ok ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "tl_halo_max")) {
		*value = c->tt_halo_max;
		return MF_OK;
	}
	return fail(c, MF_ERR_ARG, "unknown option '%s'", key);
}

MF_API mf_status mf_set_monitor(mf_ctx* c, uint32_t capacity) {
	if (!c) return MF_ERR_ARG;
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	CK(cudaSetDevice(c->cfg.device));
	drop_graph(c);
	c->mon.free();
	c->mon_counter.free();
	c->mon_cap = capacity;
	if (!capacity) return MF_OK;
	if ((uint64_t)capacity * c->bodies.size() * 4 > (1ull << 32)) return fail(c, MF_ERR_CAPACITY, "monitor too large");
	CK(c->mon.alloc((size_t)capacity * c->bodies.size() * 4));
	CK(c->mon_counter.alloc(1));
	CK(cudaMemset(c->mon_counter.p, 0, 4));
	return MF_OK;
}

MF_API mf_status mf_get_monitor(mf_ctx* c, float* out, uint32_t* rows) {
	if (!c || !rows) return MF_ERR_ARG;
	if (!c->mon_cap) return fail(c, MF_ERR_STATE, "monitor not enabled");
	uint32_t cnt = 0;
	CK(cudaMemcpyAsync(&cnt, c->mon_counter.p, 4, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	*rows = cnt < c->mon_cap ? cnt : c->mon_cap;
	if (out) CK(cudaMemcpy(out, c->mon.p, (size_t)(*rows) * c->bodies.size() * 4 * 4, cudaMemcpyDeviceToHost));
	return MF_OK;
}

MF_API mf_status mf_get_stream(mf_ctx* c, void** stream) {
	if (!c || !stream) return MF_ERR_ARG;
	*stream = (void*)c->stream;
	return MF_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ state I/O
// VTK files in the reference's legacy ASCII layout (vtk_writer.h:27-127) and exact
// binary checkpoints.  A dump first copies the state device-to-device into a snapshot
// (stream-ordered after the steps already issued, ~64 B per particle), then a host
// thread copies the snapshot out on its own stream and writes the file, so the caller
// can keep stepping.
namespace {

const char CKPT_MAGIC[8] = {'M', 'F', 'C', 'K', 'P', 'T', '1', 0};

// bytes per row of the snapshot: x y vx vy fcx fcy FP64; rho S FP64 or (mixed) FP32
size_t io_row_bytes(const mf_ctx* c) { return 6 * 8 + 4 * (c->mixed ? 4 : 8); }

mf_status io_join(mf_ctx* c) {
	if (c->io_thread.joinable()) c->io_thread.join();
	mf_status st = c->io_status;
	if (st != MF_OK) {
		c->err = c->io_err;
		c->io_status = MF_OK;
	}
	return st;
}

struct IoBody {
	uint32_t n;
	double time, rho0;
	const std::vector<double>* h;
};

// Writes the snapshot copied to host memory `hb` (layout: per field, all rows).
mf_status io_write(const char* path, int kind, int method, int precision, bool mixed, uint32_t n_total,
                   const std::vector<IoBody>& bodies, const std::vector<uint32_t>& offs, const unsigned char* hb,
                   std::string& err) {
	const double* f64[6];  // x y vx vy fcx fcy
	for (int q = 0; q < 6; q++) f64[q] = reinterpret_cast<const double*>(hb) + (size_t)q * n_total;
	const unsigned char* rest = hb + 6 * 8 * (size_t)n_total;  // rho Sxx Sxy Syy
	auto rs = [&](int q, uint32_t i, double rho0) -> double {
		if (mixed) return (double)reinterpret_cast<const float*>(rest)[(size_t)q * n_total + i] + (q == 0 ? rho0 : 0.);
		return reinterpret_cast<const double*>(rest)[(size_t)q * n_total + i];
	};
	if (kind == MF_DUMP_VTK) {
		// the host writer takes FP64 arrays per body
		std::vector<std::vector<double>> rho(bodies.size()), sxx(bodies.size()), sxy(bodies.size()), syy(bodies.size());
		std::vector<mf_vtk_body> vbs(bodies.size());
		for (size_t b = 0; b < bodies.size(); b++) {
			uint32_t o = offs[b], n = bodies[b].n;
			rho[b].resize(n); sxx[b].resize(n); sxy[b].resize(n); syy[b].resize(n);
			for (uint32_t i = 0; i < n; i++) {
				rho[b][i] = rs(0, o + i, bodies[b].rho0);
				sxx[b][i] = rs(1, o + i, 0.);
				sxy[b][i] = rs(2, o + i, 0.);
				syy[b][i] = rs(3, o + i, 0.);
			}
			vbs[b] = mf_vtk_body{n, 0, f64[0] + o, f64[1] + o, bodies[b].h->data(), rho[b].data(), sxx[b].data(),
			                     sxy[b].data(), syy[b].data(), f64[2] + o, f64[3] + o};
		}
		mf_status st = mf_vtk_write(path, vbs.data(), (uint32_t)vbs.size());
		if (st != MF_OK) err = std::string("cannot write ") + path;
		return st;
	}
	FILE* fp = fopen(path, "wb");
	if (!fp) {
		err = std::string("cannot open ") + path;
		return MF_ERR_ARG;
	}
	// checkpoint: magic, method, precision, bodies; per body n, time, then its rows of
	// x y vx vy (FP64), rho Sxx Sxy Syy (FP64, or the mixed form's FP32 with rho - rho0),
	// fcx fcy (FP64)
	bool ok = fwrite(CKPT_MAGIC, 1, 8, fp) == 8;
	uint32_t hdr[3] = {(uint32_t)method, (uint32_t)precision, (uint32_t)bodies.size()};
	ok = ok && fwrite(hdr, 4, 3, fp) == 3;
	const size_t es = mixed ? 4 : 8;
	for (size_t b = 0; b < bodies.size() && ok; b++) {
		uint32_t o = offs[b], n = bodies[b].n;
		ok = ok && fwrite(&n, 4, 1, fp) == 1 && fwrite(&bodies[b].time, 8, 1, fp) == 1;
		for (int q = 0; q < 4 && ok; q++) ok = fwrite(f64[q] + o, 8, n, fp) == n;
		for (int q = 0; q < 4 && ok; q++) ok = fwrite(rest + ((size_t)q * n_total + o) * es, es, n, fp) == n;
		for (int q = 4; q < 6 && ok; q++) ok = fwrite(f64[q] + o, 8, n, fp) == n;
	}
	ok = (fclose(fp) == 0) && ok;
	if (!ok) {
		err = std::string("cannot write ") + path;
		return MF_ERR_ARG;
	}
	return MF_OK;
}

}  // namespace

extern "C" {

MF_API mf_status mf_vtk_write(const char* path, const mf_vtk_body* bodies, uint32_t n_bodies) {
	if (!path || (n_bodies && !bodies)) return MF_ERR_ARG;
	uint64_t tot = 0;
	for (uint32_t b = 0; b < n_bodies; b++) {
		const mf_vtk_body& v = bodies[b];
		if (v.n && !(v.x && v.y && v.h && v.rho && v.Sxx && v.Sxy && v.Syy && v.vx && v.vy)) return MF_ERR_ARG;
		tot += v.n;
	}
	if (tot > 0x7fffffffull) return MF_ERR_CAPACITY;
	FILE* fp = fopen(path, "w+");
	if (!fp) return MF_ERR_ARG;
	const unsigned nt = (unsigned)tot;
	fprintf(fp, "# vtk DataFile Version 2.0\n");
	fprintf(fp, "mfree iwf\n");
	fprintf(fp, "ASCII\n");
	fprintf(fp, "\n");
	fprintf(fp, "DATASET UNSTRUCTURED_GRID\n");
	fprintf(fp, "POINTS %d float\n", nt);
	for (uint32_t b = 0; b < n_bodies; b++)
		for (uint32_t i = 0; i < bodies[b].n; i++) fprintf(fp, "%f %f %f\n", bodies[b].x[i], bodies[b].y[i], 0.);
	fprintf(fp, "\n");
	fprintf(fp, "CELLS %d %d\n", nt, 2 * nt);
	for (unsigned i = 0; i < nt; i++) fprintf(fp, "%d %d\n", 1, i);
	fprintf(fp, "\n");
	fprintf(fp, "CELL_TYPES %d\n", nt);
	for (unsigned i = 0; i < nt; i++) fprintf(fp, "%d\n", 1);
	fprintf(fp, "\n");
	fprintf(fp, "POINT_DATA %d\n", nt);
	const char* names[5] = {"h", "density", "Sxx", "Sxy", "Syy"};
	for (int k = 0; k < 5; k++) {
		fprintf(fp, "SCALARS %s float 1\n", names[k]);
		fprintf(fp, "LOOKUP_TABLE default\n");
		for (uint32_t b = 0; b < n_bodies; b++) {
			const double* a[5] = {bodies[b].h, bodies[b].rho, bodies[b].Sxx, bodies[b].Sxy, bodies[b].Syy};
			for (uint32_t i = 0; i < bodies[b].n; i++) fprintf(fp, "%f\n", a[k][i]);
		}
		fprintf(fp, "\n");
	}
	fprintf(fp, "VECTORS velocity float\n");
	for (uint32_t b = 0; b < n_bodies; b++)
		for (uint32_t i = 0; i < bodies[b].n; i++) fprintf(fp, "%f %f %f\n", bodies[b].vx[i], bodies[b].vy[i], 0.);
	fprintf(fp, "\n");
	return fclose(fp) == 0 ? MF_OK : MF_ERR_ARG;
}

MF_API mf_status mf_dump_async(mf_ctx* c, const char* path, int32_t kind) {
	if (!c || !path || (kind != MF_DUMP_VTK && kind != MF_DUMP_CHECKPOINT)) return MF_ERR_ARG;
	if (kind == MF_DUMP_CHECKPOINT && (c->cfg.method == MF_METHOD_TL_WEAK || c->cfg.method == MF_METHOD_UL_WEAK))
		return fail(c, MF_ERR_STATE, "checkpoints cover updated- and total-Lagrangian bodies (not the weak form's Gauss points)");
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = contact_flush(c)) != MF_OK) return st;
	if ((st = io_join(c)) != MF_OK) return st;  // one dump in flight at a time
	CK(cudaSetDevice(c->cfg.device));
	const uint32_t n = c->n_total;
	const size_t bytes = io_row_bytes(c) * (size_t)n;
	if (c->io_dev.n < bytes) {
		c->io_dev.free();
		CK(c->io_dev.alloc(bytes));
	}
	if (c->io_host_bytes < bytes) {
		if (c->io_host) cudaFreeHost(c->io_host);
		c->io_host = nullptr;
		c->io_host_bytes = 0;
		CK(cudaMallocHost(&c->io_host, bytes));
		c->io_host_bytes = bytes;
	}
	if (!c->io_stream) CK(cudaStreamCreateWithFlags(&c->io_stream, cudaStreamNonBlocking));
	if (!c->io_ready) CK(cudaEventCreateWithFlags(&c->io_ready, cudaEventDisableTiming));
	// snapshot on the simulation stream, after every step already issued
	unsigned char* d = c->io_dev.p;
	const double* src64[6] = {c->sd[0][0].p, c->sd[0][1].p, c->sd[0][2].p, c->sd[0][3].p, c->fcx.p, c->fcy.p};
	for (int q = 0; q < 6; q++) CK(cudaMemcpyAsync(d + (size_t)q * 8 * n, src64[q], 8 * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
	unsigned char* rest = d + 6 * 8 * (size_t)n;
	for (int q = 0; q < 4; q++) {
		if (c->mixed)
			CK(cudaMemcpyAsync(rest + (size_t)q * 4 * n, c->sf[0][q].p, 4 * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
		else
			CK(cudaMemcpyAsync(rest + (size_t)q * 8 * n, c->sd[0][4 + q].p, 8 * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
	}
	CK(cudaEventRecord(c->io_ready, c->stream));
	// what the writer needs from the host side, captured now
	std::vector<IoBody> bodies;
	std::vector<uint32_t> offs;
	for (auto& b : c->bodies) {
		bodies.push_back(IoBody{b.n, b.time, b.sd.rho0, &b.in[6]});
		offs.push_back(b.off);
	}
	std::string p(path);
	int method = c->cfg.method, prec = c->cfg.precision, dev = c->cfg.device;
	bool mixed = c->mixed;
	c->io_status = MF_OK;
	c->io_thread = std::thread([c, p, kind, method, prec, dev, mixed, n, bytes, bodies, offs]() {
		cudaError_t e = cudaSetDevice(dev);
		if (e == cudaSuccess) e = cudaStreamWaitEvent(c->io_stream, c->io_ready, 0);
		if (e == cudaSuccess) e = cudaMemcpyAsync(c->io_host, c->io_dev.p, bytes, cudaMemcpyDeviceToHost, c->io_stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(c->io_stream);
		if (e != cudaSuccess) {
			c->io_err = std::string("state dump: ") + cudaGetErrorString(e);
			c->io_status = MF_ERR_CUDA;
			return;
		}
		std::string err;
		mf_status s2 = io_write(p.c_str(), kind, method, prec, mixed, n, bodies, offs, c->io_host, err);
		if (s2 != MF_OK) {
			c->io_err = err;
			c->io_status = s2;
		}
	});
	return MF_OK;
}

MF_API mf_status mf_dump_wait(mf_ctx* c) {
	if (!c) return MF_ERR_ARG;
	return io_join(c);
}

MF_API mf_status mf_write_vtk(mf_ctx* c, const char* path) {
	mf_status st = mf_dump_async(c, path, MF_DUMP_VTK);
	return st != MF_OK ? st : mf_dump_wait(c);
}

MF_API mf_status mf_checkpoint_save(mf_ctx* c, const char* path) {
	mf_status st = mf_dump_async(c, path, MF_DUMP_CHECKPOINT);
	return st != MF_OK ? st : mf_dump_wait(c);
}

MF_API mf_status mf_checkpoint_load(mf_ctx* c, const char* path) {
	if (!c || !path) return MF_ERR_ARG;
	if (c->cfg.method == MF_METHOD_TL_WEAK || c->cfg.method == MF_METHOD_UL_WEAK)
		return fail(c, MF_ERR_STATE, "checkpoints cover updated- and total-Lagrangian bodies (not the weak form's Gauss points)");
	mf_status st = finalize(c);
	if (st != MF_OK) return st;
	if ((st = io_join(c)) != MF_OK) return st;
	c->contact_pending = false;  // the checkpoint brings the forces of its positions
	FILE* fp = fopen(path, "rb");
	if (!fp) return fail(c, MF_ERR_ARG, "cannot open %s", path);
	char magic[8];
	uint32_t hdr[3];
	bool ok = fread(magic, 1, 8, fp) == 8 && !memcmp(magic, CKPT_MAGIC, 8) && fread(hdr, 4, 3, fp) == 3;
	if (!ok || hdr[0] != (uint32_t)c->cfg.method || hdr[1] != (uint32_t)c->cfg.precision || hdr[2] != c->bodies.size()) {
		fclose(fp);
		return fail(c, MF_ERR_ARG, "%s is not a checkpoint of this context's method, precision and bodies", path);
	}
	CK(cudaSetDevice(c->cfg.device));
	const bool tl = c->cfg.method == MF_METHOD_TL || c->cfg.method == MF_METHOD_COROT ||
	                c->cfg.method == MF_METHOD_POTENTIAL;
	const size_t es = c->mixed ? 4 : 8;
	std::vector<double> times(c->bodies.size());
	std::vector<unsigned char> buf;
	for (size_t b = 0; b < c->bodies.size(); b++) {
		HostBody& B = c->bodies[b];
		uint32_t n = 0;
		ok = fread(&n, 4, 1, fp) == 1 && n == B.n && fread(&times[b], 8, 1, fp) == 1;
		buf.resize((size_t)n * (6 * 8 + 4 * es));
		ok = ok && fread(buf.data(), 1, buf.size(), fp) == buf.size();
		if (!ok) {
			fclose(fp);
			return fail(c, MF_ERR_ARG, "%s: body %zu does not match (particle count or truncated file)", path, b);
		}
		const unsigned char* q0 = buf.data();
		for (int q = 0; q < 4; q++) {  // x y vx vy
			CK(cudaMemcpy(c->sd[0][q].p + B.off, q0 + (size_t)q * 8 * n, 8 * (size_t)n, cudaMemcpyHostToDevice));
			if (tl) CK(cudaMemcpy(c->sd[2][q].p + B.off, q0 + (size_t)q * 8 * n, 8 * (size_t)n, cudaMemcpyHostToDevice));
		}
		const unsigned char* r0 = q0 + 4 * 8 * (size_t)n;
		for (int q = 0; q < 4; q++) {  // rho Sxx Sxy Syy, in the context's own representation
			const unsigned char* src = r0 + (size_t)q * es * n;
			if (c->mixed) {
				CK(cudaMemcpy(c->sf[0][q].p + B.off, src, 4 * (size_t)n, cudaMemcpyHostToDevice));
				if (tl) CK(cudaMemcpy(c->sf[2][q].p + B.off, src, 4 * (size_t)n, cudaMemcpyHostToDevice));
			} else {
				CK(cudaMemcpy(c->sd[0][4 + q].p + B.off, src, 8 * (size_t)n, cudaMemcpyHostToDevice));
				if (tl) CK(cudaMemcpy(c->sd[2][4 + q].p + B.off, src, 8 * (size_t)n, cudaMemcpyHostToDevice));
			}
		}
		const unsigned char* f0 = r0 + 4 * es * (size_t)n;
		CK(cudaMemcpy(c->fcx.p + B.off, f0, 8 * (size_t)n, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->fcy.p + B.off, f0 + 8 * (size_t)n, 8 * (size_t)n, cudaMemcpyHostToDevice));
	}
	fclose(fp);
	for (size_t b = 0; b < c->bodies.size(); b++) {
		c->bodies[b].time = times[b];
		CK(cudaMemcpy(reinterpret_cast<unsigned char*>(c->params.p) + b * sizeof(BodyParams) + offsetof(BodyParams, time),
		              &times[b], 8, cudaMemcpyHostToDevice));
	}
	c->tl_recs_valid = false;  // mixed TL: re-pack the records from the loaded state
	if ((st = tl_prepack(c)) != MF_OK) return st;
	CK(cudaStreamSynchronize(c->stream));
	return MF_OK;
}

}  // extern "C"
