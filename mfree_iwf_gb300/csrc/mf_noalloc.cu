// mf_ul_step_noalloc: the updated-Lagrangian RK4 step for callers that cannot
// allocate device memory.
//
// Some callers must not allocate on the device after start-up: applications that
// reserve all GPU memory up front in their own pools and forbid allocations later,
// and plug-ins that run inside another framework's stream and must not trigger the
// implicit device-wide synchronisation of cudaMalloc/cudaFree.  A context
// (mf_create) allocates all of its buffers, so those callers use this entry point
// instead: the caller passes the particle arrays (device pointers, updated in
// place), and every buffer of the step -- cell grid, sort keys and radix-sort
// workspace, cell-ordered records, RK4 accumulators and stage state, status word --
// lives in one file-scope device array of fixed size, g_noalloc_scratch below.
//
// Limits and sharing:
//   * at most MF_NOALLOC_MAX_PARTICLES particles in one call (larger n is rejected
//     with MF_ERR_CAPACITY);
//   * the array is allocated once per device when the library's device code is
//     loaded there and is held until the process exits;
//   * every call on a device uses the same array and leaves its contents behind for
//     the next call; the parts that must start from zero (contact forces, body index,
//     status word) are cleared by each call.  Calls whose work overlaps on the GPU
//     (different streams, or different host threads) race on the array and give
//     undefined results: serialise them.
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and queries the sort workspace size; make that first
//     call before any stream capture begins.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/mfree_gb300.h"
#include "mf_kernels.h"

using namespace mfk_host;

namespace {

constexpr uint32_t kMaxN = MF_NOALLOC_MAX_PARTICLES;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// byte offsets of the parts of the scratch array (n = kMaxN)
constexpr size_t OFF_STATUS = 0;
constexpr size_t OFF_PARAMS = align_up(OFF_STATUS + sizeof(DevStatusH));
constexpr size_t OFF_GEOM = align_up(OFF_PARAMS + sizeof(BodyParams));
constexpr size_t OFF_BBOX = align_up(OFF_GEOM + sizeof(Geom));
constexpr size_t OFF_TOTAL = align_up(OFF_BBOX + 6 * sizeof(unsigned long long));
constexpr size_t OFF_KEYS = align_up(OFF_TOTAL + sizeof(uint32_t));
constexpr size_t OFF_KEYS_SORTED = align_up(OFF_KEYS + 4ull * kMaxN);
constexpr size_t OFF_PERM_IN = align_up(OFF_KEYS_SORTED + 4ull * kMaxN);
constexpr size_t OFF_PERM = align_up(OFF_PERM_IN + 4ull * kMaxN);
constexpr size_t OFF_CELLS = align_up(OFF_PERM + 4ull * kMaxN);
constexpr size_t OFF_BODY_OF = align_up(OFF_CELLS + 4ull * (kMaxN + 2));
constexpr size_t OFF_REC_BODY = align_up(OFF_BODY_OF + 4ull * kMaxN);
constexpr size_t OFF_FC = align_up(OFF_REC_BODY + 4ull * kMaxN);          // fcx, fcy
constexpr size_t OFF_ACC = align_up(OFF_FC + 2 * 8ull * kMaxN);           // 8 fields
constexpr size_t OFF_ST = align_up(OFF_ACC + 8 * 8ull * kMaxN);           // 8 fields
constexpr size_t OFF_REC = align_up(OFF_ST + 8 * 8ull * kMaxN);           // 128 B per row
constexpr size_t OFF_SORT_TMP = align_up(OFF_REC + 128ull * kMaxN);
constexpr size_t SORT_TMP_BYTES = 1u << 20;
constexpr size_t SCRATCH_BYTES = OFF_SORT_TMP + SORT_TMP_BYTES;

// The scratch of every mf_ul_step_noalloc call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

struct DeviceSetup {
	bool done = false;
	unsigned char* base = nullptr;
	size_t sort_tmp_needed = 0;
};
std::mutex g_mutex;
DeviceSetup g_setup[64];

// Once per device, with that device current: the device address of the array.
mf_status setup_device(int dev, DeviceSetup*& out) {
	if (dev < 0 || dev >= 64) return MF_ERR_ARG;
	std::lock_guard<std::mutex> lock(g_mutex);
	DeviceSetup& s = g_setup[dev];
	if (!s.done) {
		void* p = nullptr;
		if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MF_ERR_CUDA;
		s.base = static_cast<unsigned char*>(p);
		int bits = 1;
		while (bits < 32 && (1ull << bits) < (uint64_t)kMaxN + 2) bits++;
		s.sort_tmp_needed = mf_strict::ul_sort_tmp_bytes(kMaxN, bits);
		if (s.sort_tmp_needed > SORT_TMP_BYTES) return MF_ERR_CAPACITY;
		s.done = true;
	}
	out = &s;
	return MF_OK;
}

inline uint32_t abit(int a) { return 1u << a; }

}  // namespace

extern "C" MF_API mf_status mf_ul_step_noalloc(const mf_device_body* body, const mf_sim_data* sd, double dt,
                                                const int32_t* actions, uint32_t n_actions, int32_t nsteps,
                                                void* stream) {
	if (!body || !sd || (!actions && n_actions)) return MF_ERR_ARG;
	if (nsteps < 0 || !(dt > 0.)) return MF_ERR_ARG;
	if (body->n == 0) return MF_ERR_ARG;
	if (body->n > kMaxN) return MF_ERR_CAPACITY;
	if (!body->x || !body->y || !body->vx || !body->vy || !body->rho || !body->Sxx || !body->Sxy || !body->Syy ||
	    !body->m || !body->h || !body->quad_weight)
		return MF_ERR_ARG;
	// the action list: an ascending subsequence of the rings_monaghan list (rings.cpp:86-96)
	uint32_t flags = 0;
	int prev = 0;
	for (uint32_t k = 0; k < n_actions; k++) {
		int a = actions[k];
		if (a < MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS || a > MF_CONTMECH_ADVECTION || a <= prev) return MF_ERR_PIPELINE;
		prev = a;
		flags |= abit(a);
	}
	if ((flags & abit(MF_CONTMECH_MOMENTUM_UL)) && !(flags & abit(MF_DERIVE_STRESS_MONAGHAN))) return MF_ERR_PIPELINE;
	if ((flags & (abit(MF_MATERIAL_STRESS_RATE_JAUMANN) | abit(MF_CONTMECH_CONTINUITY))) &&
	    !(flags & abit(MF_DERIVE_VELOCITY)))
		return MF_ERR_PIPELINE;

	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return MF_ERR_NO_DEVICE;
	DeviceSetup* S = nullptr;
	mf_status st = setup_device(dev, S);
	if (st != MF_OK) return st;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	unsigned char* B = S->base;
	uint32_t n = body->n;

	// per-body constants, as mf_add_body derives them (simulation_data.cpp:32-47)
	BodyParams p{};
	double nu = sd->nu, E = sd->E, rho0 = sd->rho0;
	double G = E / (2. * (1. + nu));
	double K = 2.0 * G * (1 + nu) / (3 * (1 - 2 * nu));
	double c0 = sqrt(K / rho0);
	p.K = K; p.G = G; p.rho0 = rho0; p.c0sq = c0 * c0;
	p.E = E; p.nu = nu; p.D = E / (1 - nu * nu);
	p.wdeltap = sd->mghn_wdeltap; p.corr_exp = sd->mghn_corr_exp; p.mghn_eps = sd->mghn_eps;
	p.alpha = sd->artvisc_alpha; p.beta = sd->artvisc_beta; p.eta = sd->artvisc_eta; p.xsph_eps = sd->xsph_eps;
	p.dt = dt; p.off = 0; p.n = n;

	// clear what must start at zero; the rest is overwritten before it is read
	DevStatusH zero_status{0u, 0xffffffffu};
	if (cudaMemcpyAsync(B + OFF_STATUS, &zero_status, sizeof zero_status, cudaMemcpyHostToDevice, s) != cudaSuccess ||
	    cudaMemcpyAsync(B + OFF_PARAMS, &p, sizeof p, cudaMemcpyHostToDevice, s) != cudaSuccess ||
	    cudaMemsetAsync(B + OFF_BODY_OF, 0, 4ull * n, s) != cudaSuccess ||
	    cudaMemsetAsync(B + OFF_FC, 0, 2 * 8ull * kMaxN, s) != cudaSuccess)
		return MF_ERR_CUDA;

	ULArgs a{};
	a.n_total = n;
	a.n_bodies = 1;
	a.flags = flags;
	a.max_nbh = 200;  // MAX_NBH, particle.h:31
	a.strict_grid = 1;
	a.nbh_eps = 1e-6;  // grid.h:157
	a.params = reinterpret_cast<const BodyParams*>(B + OFF_PARAMS);
	a.geom = reinterpret_cast<Geom*>(B + OFF_GEOM);
	a.bbox = reinterpret_cast<unsigned long long*>(B + OFF_BBOX);
	a.total_cells = reinterpret_cast<uint32_t*>(B + OFF_TOTAL);
	a.body_of = reinterpret_cast<const uint32_t*>(B + OFF_BODY_OF);
	a.m = body->m; a.h = body->h; a.qw0 = body->quad_weight;
	a.fcx = reinterpret_cast<const double*>(B + OFF_FC);
	a.fcy = a.fcx + kMaxN;
	a.base = StateSoA{body->x, body->y, body->vx, body->vy, body->rho, body->Sxx, body->Sxy, body->Syy,
	                  nullptr, nullptr, nullptr, nullptr};
	double* acc = reinterpret_cast<double*>(B + OFF_ACC);
	double* stg = reinterpret_cast<double*>(B + OFF_ST);
	a.acc = StateSoA{acc, acc + kMaxN, acc + 2 * kMaxN, acc + 3 * kMaxN, acc + 4 * kMaxN, acc + 5 * kMaxN,
	                 acc + 6 * kMaxN, acc + 7 * kMaxN, nullptr, nullptr, nullptr, nullptr};
	a.st = StateSoA{stg, stg + kMaxN, stg + 2 * kMaxN, stg + 3 * kMaxN, stg + 4 * kMaxN, stg + 5 * kMaxN,
	                stg + 6 * kMaxN, stg + 7 * kMaxN, nullptr, nullptr, nullptr, nullptr};
	a.keys = reinterpret_cast<uint32_t*>(B + OFF_KEYS);
	a.keys_sorted = reinterpret_cast<uint32_t*>(B + OFF_KEYS_SORTED);
	a.perm_in = reinterpret_cast<uint32_t*>(B + OFF_PERM_IN);
	a.perm = reinterpret_cast<uint32_t*>(B + OFF_PERM);
	a.cell_start = reinterpret_cast<uint32_t*>(B + OFF_CELLS);
	a.rec = B + OFF_REC;
	a.rec_body = reinterpret_cast<uint32_t*>(B + OFF_REC_BODY);
	a.sort_tmp = B + OFF_SORT_TMP;
	a.sort_tmp_bytes = S->sort_tmp_needed;
	int bits = 1;
	while (bits < 32 && (1ull << bits) < (uint64_t)n + 2) bits++;
	a.sort_bits = bits;
	a.status = reinterpret_cast<DevStatusH*>(B + OFF_STATUS);

	for (int32_t k = 0; k < nsteps; k++)
		for (uint32_t stage = 0; stage < 4; stage++) {
			a.stage = stage;
			if (mf_strict::ul_stage(a, false, s) != cudaSuccess) return MF_ERR_CUDA;
		}
	DevStatusH hs{};
	if (cudaMemcpyAsync(&hs, B + OFF_STATUS, sizeof hs, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
	    cudaStreamSynchronize(s) != cudaSuccess)
		return MF_ERR_CUDA;
	if (hs.flags & 8u) return MF_ERR_NONFINITE;
	if (hs.flags & 4u) return MF_ERR_GRID;
	if (hs.flags & 1u) return MF_ERR_NBH_OVERFLOW;
	if (hs.flags & 2u) return MF_ERR_NO_NEIGHBOR;
	return hs.flags ? MF_ERR_CUDA : MF_OK;
}
