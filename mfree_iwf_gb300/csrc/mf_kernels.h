// Host-visible declarations of the kernel launchers.  Each launcher exists in
// two namespaces compiled from the same sources: mf_strict (FP64 without FMA
// contraction, the parity form) and mf_fast (FP64 and mixed precision with
// contraction).  All launchers enqueue on the given stream and never synchronise.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace mfk_host {

// Action flags of a fused pipeline (bit i = action id i of mf_action).
inline uint32_t bit(int a) { return 1u << a; }
// Actions with ids of 32 and above take flag bits that their method's pipeline leaves
// free: the Godunov pair actions (updated-Lagrangian only) the bits of two
// total-Lagrangian actions, the elastic-potential forces bit 0.
constexpr uint32_t FLAG_GODUNOV_CONTINUITY = 1u << 12;
constexpr uint32_t FLAG_GODUNOV_MOMENTUM = 1u << 13;
constexpr uint32_t FLAG_POTENTIAL = 1u << 0;
// The weak updated-Lagrangian form's own actions (ids 35-40) take the bits of the
// total-Lagrangian actions 12-17, which its pipeline never holds.
constexpr uint32_t FLAG_UW_RIEMANN_GP = 1u << 12;
constexpr uint32_t FLAG_UW_STRESS = 1u << 13;
constexpr uint32_t FLAG_UW_VEL_WEAK = 1u << 14;
constexpr uint32_t FLAG_UW_MOMENTUM_W = 1u << 15;
constexpr uint32_t FLAG_UW_INTERP = 1u << 16;
constexpr uint32_t FLAG_UW_ADVECTION_GP = 1u << 17;

// Per-body constants (simulation_data.h:25-99 plus the body's dt), device copy.
struct BodyParams {
	double K, G, rho0, c0sq;        // c0sq = c0*c0 with c0 = sqrt(K/rho0) (material.h:37-44)
	double E, nu, D;                // D = E/(1-nu^2) (material.h:136)
	double wdeltap, corr_exp, mghn_eps;
	double alpha, beta, eta, xsph_eps;
	double dt, time;
	uint32_t off, n;                // particle rows [off, off+n)
	uint32_t pad0, pad1;
	// FP32 copies for the mixed passes (a conversion from FP64 runs on the FP64 pipe)
	float fK, fG, frho0, fc0sq, fD, fnu, falpha, fbeta, feta2, fdt;
	float fwdp1, fcorr_exp, fxsph_eps, fmghn_eps;  // fwdp1 = 1 / wdeltap (0 when wdeltap <= 0)
};

// Per-body cell geometry of one derivative evaluation (grid.h:83-115).
struct Geom {
	double bbmin_x, bbmin_y, dx;
	double slack;  // mixed form: how far a particle may move within the step
	uint32_t nx, ny, num_cell, cell_off;
	uint32_t span;  // stencil half-width in cells: 1 (cells of 2 h_max [+ 2 slack]) or 2 (mixed: half-size cells)
	uint32_t pad;
};

struct DevStatusH {
	uint32_t flags;
	uint32_t first_index;
};

// State arrays of a body set (rows of all bodies concatenated).
// FP64 forms: every pointer is double.  Mixed form: x, y, vx, vy are double,
// rho and the stresses are float (the *_f pointers).
struct StateSoA {
	double *x, *y, *vx, *vy, *rho, *Sxx, *Sxy, *Syy;
	float *rho_f, *Sxx_f, *Sxy_f, *Syy_f;
};

struct ULArgs {
	uint32_t n_total, n_bodies, stage;    // stage 0..3
	uint32_t flags;                       // action bits
	uint32_t max_nbh;                     // neighbour capacity (0 = unchecked)
	uint32_t strict_grid;                 // 1: rebuild the reference grid at this stage
	double nbh_eps;
	const BodyParams* params;             // device
	Geom* geom;                           // device, per body
	unsigned long long* bbox;             // device, 6 per body
	uint32_t* total_cells;                // device scalar
	const uint32_t* body_of;              // device, per row
	const double *m, *h, *qw0, *fcx, *fcy;  // constants (home order)
	StateSoA base, acc, st;               // RK4 arrays (home order)
	uint32_t *keys, *keys_sorted, *perm_in, *perm;  // sort buffers
	uint32_t* cell_start;                 // capacity cell_cap + 1
	uint32_t cell_cap;                    // most cells over all bodies (0: n_total + 1)
	void* rec;                            // cell-ordered gathered records
	uint32_t* rec_body;                   // body of each cell-ordered row
	void* sort_tmp;
	size_t sort_tmp_bytes;
	int sort_bits;
	mfk_host::DevStatusH* status;
	cudaEvent_t ev_pair0, ev_pair1;       // optional timing of the pair kernel
	// launch shape of the pair kernel (autotuned): rows per block, and, when
	// persistent, a fixed grid whose blocks pull chunks of `chunk` blocks' worth of
	// rows from the atomic counter `work` until all rows are done
	uint32_t block, persistent, grid, chunk;
	uint32_t split;  // mixed, plain grid: threads per row of the pair pass (1, 4 or 8)
	uint32_t* work;
	// per-body failure words (ERR_* bits), device; nullptr: an error of any row fails the
	// whole step.  When set, a row's error marks its body failed instead, and a failed
	// body's rows are left out of the grid and the pair pass from then on (frozen).
	uint32_t* failed;
	// mixed: the pair pass of stages 0-2 also writes each row's record of the next stage
	// into rec_next (the cell order holds for the whole step), and the next stage skips
	// the gather
	void* rec_next;
	uint32_t write_recs, skip_gather;
};

// Neighbour search of the total-Lagrangian set-up (find_neighbors,
// neighbor_search.h:50-147): query points "to" against particles "from".
struct TLSearchArgs {
	uint32_t n_from, n_to;
	const double *fx, *fy, *tx, *ty;
	const uint32_t *from_body, *to_body;
	const Geom* geom;          // per body, cell >= search radius
	uint32_t total_cells;
	double h, eps;
	uint32_t max_nbh;
	uint32_t *keys, *keys_sorted, *vals, *perm, *cell_start;
	void* sort_tmp;
	size_t sort_tmp_bytes;
	int sort_bits;
	uint32_t* count;           // pass 0 output
	const uint32_t* off;       // pass 1 input (exclusive scan of count)
	uint32_t* nbr;             // pass 1 output
	uint32_t manhattan;        // 1: |dx| < 2h + 1e-6 and |dy| < 2h + 1e-6 (neighbor_search.h:43-48)
	void* status;
};

// One total-Lagrangian stage over all bodies.
struct TLArgs {
	uint32_t n_total, n_bodies, stage, flags;
	const BodyParams* params;
	const uint32_t* body_of;
	const double *X, *Y, *m, *h, *qw0, *fcx, *fcy;
	const void *qw32, *m32, *h32;       // mixed form: float copies of the constants
	StateSoA base, acc, st, nxt;         // st: this stage's state, nxt: the next stage's
	// neighbour lists in sliced-ELL form: rows in slices of 32, entry k of row r of
	// slice s at sl_off[s] + 32*k + (r % 32); cnt[r] entries per row, ascending j
	const uint32_t* sl_off;
	const uint16_t* cnt;
	const uint32_t* snbr;
	const void* sw;                      // corrected gradient per pair: double2 (FP64 forms) / float2 times m_j (mixed)
	const void* swA;                     // mixed: the gradient times the neighbour's quad weight (pass A)
	void *P, *dA, *c;                    // per-stage scratch (FP64 forms)
	const void* sW;                      // corotational: kernel value W per pair (double, sliced ELL);
	                                     // potential: grad W of the reverse pair (double2, sliced ELL)
	void* R;                             // corotational: per row double4 {cos, sin, m, 0} of the rotation
	void* av;                            // corotational / potential: per row two double4 records
	                                     // {x, y, vx, vy} and {h, rho, c, m} for the viscosity loop
	// corotational / potential, mixed form: per pair (sliced ELL) float2 gradients times
	// m_j (corotational) or plain (potential), times qw_j (pass A), X_j - X_i and m_j W_ij
	// (corotational), the reverse gradient (potential); per row float4 records:
	// displacement, position and velocity as float-float pairs, stress, rotation
	// {cos, sin, cos - 1, m}, {h, rho, c, m}
	const void *cm_sw, *cm_swA, *cm_sX, *cm_sW, *cm_swji;
	void *cm_U, *cm_X, *cm_V, *cm_P, *cm_R, *cm_H;
	void *recA, *recB;                   // mixed: per-row records: recA float4 per row; recB four float4
	                                     // field arrays of n_total (P, x, v, {h, m, rho, c})
	void* recB_out;                      // mixed: pass B writes the next stage's records here...
	uint32_t write_recs;                 // ...and into recA when set (no separate pack then)
	void* dA32;                          // mixed: rate terms (float4 per row)
	// mixed form, run walk: each row's ascending neighbour list as runs of consecutive
	// rows, one word per run (first row | (length - 1) << TL_RUN_SHIFT), in sliced ELL
	// (r_sl per slice of 32 rows, r_cnt runs per row); the passes recompute every pair's
	// corrected gradient from the reference positions as float-float pairs (XF: float4
	// {X hi, X lo, Y hi, Y lo} per row) and the row's Randles-Libersky correction
	// (G: float4 {invB00, invB10, invB01, invB11} / C).  runs == nullptr: the lists.
	const uint32_t* r_sl;
	const uint16_t* r_cnt;
	const uint32_t* runs;
	const void *XF, *G;
	uint32_t unroll;                     // run walk: 1 or 2 pairs per loop iteration; 3: one pair, pass B
	                                     // with 64 registers; 4: also pass A with 48 (all: the same results)
	const uint32_t* bc_rows;
	const double* bc_v;
	uint32_t n_bc;
	void* status;
	uint32_t block;                      // rows per block of the pair passes (autotuned)
	// mixed form, halo tiles: tile t holds positions [t*TL_TILE, (t+1)*TL_TILE) of a
	// space-filling-curve order (t_rows[p] = row); its halo -- every row a list of the
	// tile names -- is t_halo[t_halo_off[t] .. t_halo_off[t+1]) (ascending), staged in
	// shared memory by the pass; lists are sliced ELL over positions holding the halo
	// slot (t_loc) and the same FP32 weights as sw / swA.  t_rows == nullptr: untiled.
	const uint32_t* t_rows;
	const uint32_t* t_halo_off;
	const uint32_t* t_halo;
	const uint32_t* t_sl;
	const uint16_t* t_cnt;
	const uint16_t* t_loc;
	const void* t_sw;
	const void* t_swA;
	uint32_t n_tiles, halo_max;
	uint32_t t_ent_max;  // most list entries (sliced-ELL slots) of one tile
};
constexpr uint32_t TL_TILE = 128;
constexpr uint32_t TL_RUN_SHIFT = 27;  // runs: start rows below 2^27, lengths 1..32
constexpr uint32_t TL_RUN_MAX_ROWS = 1u << TL_RUN_SHIFT;
constexpr uint32_t TL_RUN_MAX_LEN = 32;

// One weak-form stage: particles (state x, y, vx, vy) and Gauss points (state rho,
// Sxx, Sxy, Syy in the rho/Sxx/Sxy/Syy or *_f slots of the StateSoA).
struct WeakArgs {
	uint32_t n_p, n_g, n_bodies, stage, flags, block;
	const BodyParams* params;
	const uint32_t *body_of, *gp_body;
	const double *X, *Y, *m, *qw_p, *gp_qw, *fcx, *fcy;
	const double *gp_ux, *gp_uy;  // Gauss points' own displacement x - X
	StateSoA base, acc, st;      // particles
	StateSoA gbase, gacc, gst;   // Gauss points
	// sliced-ELL lists: Gauss point -> particles (gradients), particle -> Gauss points
	// (transposed, gradients), particle -> particles (shape-function values)
	const uint32_t *g_sl, *g_snbr, *t_sl, *t_snbr, *p_sl, *p_snbr;
	const uint16_t *g_cnt, *t_cnt, *p_cnt;
	const void *g_w, *t_w, *p_w;  // double2 (FP64 forms) / float2 (mixed, pre-multiplied weights)
	void* gP;                     // nominal stress per Gauss point
	void* pack;                   // mixed: per particle u and v as float-float (2 x float4)
	const uint32_t* bc_rows;
	const double* bc_v;
	uint32_t n_bc;
	void* status;
};

// Weak updated-Lagrangian form (particle_ul_weak): particles and stress points, both
// with fixed candidate lists (ascending) and, per derivative evaluation, the
// candidates inside the neighbour ellipse (mask) with their RKPM shape functions.
//
// A row's k-th candidate sits in slot start[i] + k * stride, k < cnt[i]; masks and
// shape functions share the slots.  The ellipse lists are sliced (stride 32: the 32
// rows of a slice interleaved, so the 32 rows of a warp reach their k-th slots in one
// contiguous line); element maps keep rows contiguous (stride 1).
struct SlotList {
	const uint32_t *start, *cnt, *nbr;
	uint32_t stride;
};
struct GSoA {
	double *x, *y, *rho, *Sxx, *Sxy, *Syy;
};
struct UWArgs {
	uint32_t n_p, n_g, stage, flags, block;
	const BodyParams* params;
	const uint32_t *body_of, *gbody_of;
	const double *m, *gm, *fcx, *fcy;
	double *qw_base, *gqw_base;          // quad weights of the particles / stress points
	double* qw_stage;                    // the particles' weights of this evaluation
	StateSoA base, acc, rd, wr;          // particles: this stage reads rd, writes wr
	GSoA gbase, gacc, grd, gwr;          // stress points
	SlotList pc, gc;                     // candidate lists of the particles / stress points
	uint8_t *pmask, *gmask;              // per candidate: inside this evaluation's ellipse
	double *pw, *pwx, *pwy, *gw, *gwx, *gwy;  // per candidate: shape function and gradient
	SlotList tp;                         // per particle: the stress points listing it, ascending (sliced)
	const uint32_t* tp_slot;             // their candidate slots, in tp's slots
	double* gsig;                        // per stress point: Sxx - p, Sxy, Syy - p, quad weight
	// mixed form (null otherwise): the particles' float-float velocities and weights of
	// the evaluation (qw32 + qwlo), the stress points' gsig in FP32
	const float4* vff;
	const float *qw32, *qwlo;
	float4* gsig32;
	const uint32_t* bc_of;               // per particle: index into bc_v, or ~0u
	const double* bc_v;
	void* status;
};

// Contact: boundary points of all bodies, their 32-point tiles, and the slave rows
// with the master body each one is tested against.
struct ContactArgs {
	uint32_t n_bnd, n_tiles, n_slave;
	const uint32_t *bnd_rows, *bnd_start, *bnd_len;   // per boundary point
	double4* bnd;                                       // x, y, nx, ny
	float4* bnd_ff;                                     // x, y as float-float pairs
	const uint32_t *tile_first, *tile_end;
	float4* tile_bb;
	const uint32_t *slave_rows, *slave_master;
	const double* dt;                                   // per slave row
	const uint32_t *m_tile_off, *m_tile_n;              // per body
	const double *x, *y, *m;
	double *fcx, *fcy;
};

}  // namespace mfk_host

#define MF_DECLARE_LAUNCHERS(NS)                                                                              \
	namespace NS {                                                                                           \
	size_t ul_sort_tmp_bytes(uint32_t n, int bits);                                                          \
	size_t ul_rec_bytes(bool mixed);                                                                         \
	cudaError_t ul_stage(const mfk_host::ULArgs& a, bool mixed, cudaStream_t s);                             \
	cudaError_t ul_bc(uint32_t n_bc, const uint32_t* rows, const double* v, double* vx, double* vy, cudaStream_t s); \
	cudaError_t ul_neighbors(const mfk_host::ULArgs& a, uint32_t* counts, uint32_t* idx, const uint64_t* offs, \
	                         int pass, cudaStream_t s);                                                      \
	size_t tl_sort_tmp_bytes(uint32_t n, int bits);                                                          \
	cudaError_t tl_search(const mfk_host::TLSearchArgs& a, int pass, cudaStream_t s);                        \
	cudaError_t tl_rl(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* x, const double* y, \
	                  const double* m, const double* rho, const float* rho_f, const double* h, double* wx,   \
	                  double* wy, void* g32, void* status, cudaStream_t s);                                  \
	cudaError_t tl_ref_positions(uint32_t n, const double* X, const double* Y, void* XF, cudaStream_t s);     \
	cudaError_t to_float(uint64_t n, const double* a, float* b, cudaStream_t s);                             \
	cudaError_t tl_to_sell(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* wx, const double* wy, \
	                       const uint32_t* sl_off, uint16_t* cnt, uint32_t* snbr, void* sw64, void* sw32,     \
	                       void* swA32, const double* qw, const double* mass, cudaStream_t s);                \
	cudaError_t tl_stage(const mfk_host::TLArgs& a, bool mixed, int part, cudaStream_t s);                   \
	cudaError_t tl_tile_sell(uint32_t n, const uint32_t* t_rows, const uint32_t* sl_off, const uint16_t* cnt, \
	                         const void* sw, const void* swA, const uint32_t* t_sl, uint16_t* t_cnt, void* t_sw, \
	                         void* t_swA, cudaStream_t s);                                                  \
	cudaError_t tl_tile_attrs(uint32_t halo_max, uint32_t ent_max);                                          \
	cudaError_t cr_sph(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* x, const double* y, \
	                   const double* h, double* w, double* wx, double* wy, cudaStream_t s);                 \
	cudaError_t cr_sell_wji(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* wx, const double* wy,  \
	                        const uint32_t* sl_off, void* sWji, cudaStream_t s);                                   \
	cudaError_t cr_sell_w(uint32_t n, const uint32_t* off, const uint32_t* sl_off, const double* w, double* sW, \
	                      cudaStream_t s);                                                                   \
	cudaError_t cr_stage(const mfk_host::TLArgs& a, int part, cudaStream_t s);                               \
	cudaError_t cr_mixed_lists(uint32_t n, const uint32_t* sl_off, const uint16_t* cnt, const uint32_t* snbr,   \
	                           const void* sw64, const double* sW64, int potential, const double* X,        \
	                           const double* Y, const double* m, const double* qw, void* sw, void* swA,      \
	                           void* sX, void* sW, void* swji, cudaStream_t s);                              \
	cudaError_t contact_step(const mfk_host::ContactArgs& a, cudaStream_t s);                                \
	cudaError_t weak_gauss_points(uint32_t n_elem, const uint32_t* quads, uint32_t order, const double* px,    \
	                              const double* py, double* gx, double* gy, double* gqw, double* fw,         \
	                              double* fwx, double* fwy, void* status, cudaStream_t s);                    \
	cudaError_t weak_gp_disp(uint32_t n, const double* gx, const double* gy, const double* gX, const double* gY, \
	                         double* ux, double* uy, cudaStream_t s);                                           \
	cudaError_t weak_rkpm(uint32_t n_to, const double* tx, const double* ty, const double* th,                \
	                      const uint32_t* off, const uint32_t* nbr, const double* fx, const double* fy,       \
	                      const double* fm, const double* frho, const float* frho_f, double* w, double* wx,    \
	                      double* wy, void* status, cudaStream_t s);                                          \
	cudaError_t weak_transpose(uint32_t n_p, const uint32_t* toff, const uint32_t* tnbr, const uint32_t* goff, \
	                           const uint32_t* gnbr, const double* gwx, const double* gwy, double* twx,       \
	                           double* twy, void* status, cudaStream_t s);                                    \
	cudaError_t weak_sell(uint32_t n, const uint32_t* off, const uint32_t* nbr, const double* a, const double* b, \
	                      const uint32_t* sl_off, uint16_t* cnt, uint32_t* snbr, void* out64, void* out32,     \
	                      const double* mul_row, const double* mul_nbr, cudaStream_t s);                      \
	cudaError_t weak_stage(const mfk_host::WeakArgs& a, bool mixed, int part, cudaStream_t s);               \
	cudaError_t uw_nbh(uint32_t n_to, const double* tx, const double* ty, const mfk_host::SlotList& cand,          \
	                   const double* fx, const double* fy, const double* fm, const double* frho, double* h_out,  \
	                   uint8_t* mask, double* w, double* wx, double* wy, const double* qw_src, double* qw_dst,   \
	                   const void* ff, const float* vol, void* status, cudaStream_t s);                     \
	cudaError_t uw_ff(uint32_t n, const double* x, const double* y, const double* vx, const double* vy,           \
	                  const double* m, const double* rho, const double* qw_src, double* qw_dst, void* ff,      \
	                  void* vff, float* vol, float* qw32, float* qwlo, cudaStream_t s);                     \
	cudaError_t uw_stage(const mfk_host::UWArgs& a, int part, cudaStream_t s);                                \
	}

MF_DECLARE_LAUNCHERS(mf_strict)
MF_DECLARE_LAUNCHERS(mf_fast)
