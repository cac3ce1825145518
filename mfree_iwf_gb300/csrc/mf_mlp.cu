// MLP surrogate: an ensemble of small fully connected ReLU networks with BF16 weights
// and activations and FP32 accumulation, trained with Adam on FP32 master weights.
// It maps ring-impact parameters to the solver's rebound velocity, peak von Mises
// stress and contact-force history (mfree_iwf_gb300/surrogate.py).  No counterpart in
// the reference: this is a learned screen placed in front of the solver.
//
// The forward products go through a pipelined tensor-core GEMM (k_gemm_nt: 128x64
// tiles, cp.async double buffering, ldmatrix fragments); the backward products, whose
// operands are transposed, through a simpler tiled one (k_gemm: 64x64 tiles staged
// element-wise).  Both issue mma.sync m16n8k16 (BF16 inputs, FP32 accumulators) with
// gridDim.z over the ensemble members, and fuse the bias and ReLU into the epilogue,
// which stores FP32 and/or BF16.  The layers (6 -> 256 -> 256 -> 256 -> 66, a few hundred rows per
// training batch) are too small for a TMA/tcgen05 pipeline to pay off.
//
// Training keeps the whole data set on the device.  One training step -- bootstrap
// minibatch gather (each member draws its own rows), forward, MSE, backward, Adam --
// is captured once as a CUDA graph and replayed; the step counter, learning-rate
// schedule and loss history live in device memory, so replays need no host work.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched from the driver at run time
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mfree_gb300.h"

namespace {

typedef __nv_bfloat16 bf16;

struct GemmArgs {
	int M, N, K;
	const bf16* A;
	int lda;
	long long sA;  // member strides, elements
	const bf16* B;
	int ldb;
	long long sB;
	float* C;  // FP32 output, optional
	int ldc;
	long long sC;
	bf16* Cb;  // BF16 output, optional
	int ldcb;
	long long sCb;
	const float* bias;  // per output column, optional
	long long sBias;
	int relu;
	int n_store;  // tcgen05 path: FP32 output columns stored (0: all N), any ldc
};

constexpr int BM = 64, BN = 64, BK = 32, PADK = BK + 8;  // 80-byte rows: conflict-free fragment loads

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// C[M x N] = op(A)[M x K] op(B)[K x N]
//   TA = false: A(m, k) = A[m*lda + k]   TA = true: A(m, k) = A[k*lda + m]
//   TB = false: B(k, n) = B[k*ldb + n]   TB = true: B(k, n) = B[n*ldb + k]
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
	__shared__ __align__(16) bf16 As[BM][PADK];  // [m][k]
	__shared__ __align__(16) bf16 Bs[BN][PADK];  // [n][k]
	const int z = blockIdx.z;
	const bf16* A = g.A + z * g.sA;
	const bf16* B = g.B + z * g.sB;
	const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int wm = warp >> 1, wn = warp & 1;
	const int gid = lane >> 2, tig = lane & 3;
	float acc[2][4][4];
#pragma unroll
	for (int a = 0; a < 2; a++)
#pragma unroll
		for (int b = 0; b < 4; b++)
#pragma unroll
			for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
	const bf16 zero = __float2bfloat16(0.f);
	for (int k0 = 0; k0 < g.K; k0 += BK) {
		// stage the tiles; consecutive threads walk the contiguous dimension
#pragma unroll 4
		for (int e = tid; e < BM * BK; e += 128) {
			const int mm = TA ? (e % BM) : (e / BK), kk = TA ? (e / BM) : (e % BK);
			const int m = m0 + mm, k = k0 + kk;
			bf16 v = zero;
			if (m < g.M && k < g.K) v = TA ? A[(long long)k * g.lda + m] : A[(long long)m * g.lda + k];
			As[mm][kk] = v;
		}
#pragma unroll 4
		for (int e = tid; e < BN * BK; e += 128) {
			const int nn = TB ? (e / BK) : (e % BN), kk = TB ? (e % BK) : (e / BN);
			const int n = n0 + nn, k = k0 + kk;
			bf16 v = zero;
			if (n < g.N && k < g.K) v = TB ? B[(long long)n * g.ldb + k] : B[(long long)k * g.ldb + n];
			Bs[nn][kk] = v;
		}
		__syncthreads();
#pragma unroll
		for (int ks = 0; ks < BK; ks += 16) {
			uint32_t af[2][4], bfr[4][2];
			const int c = ks + tig * 2;
#pragma unroll
			for (int mt = 0; mt < 2; mt++) {
				const int r = wm * 32 + mt * 16 + gid;
				af[mt][0] = ld_pair(&As[r][c]);
				af[mt][1] = ld_pair(&As[r + 8][c]);
				af[mt][2] = ld_pair(&As[r][c + 8]);
				af[mt][3] = ld_pair(&As[r + 8][c + 8]);
			}
#pragma unroll
			for (int nt = 0; nt < 4; nt++) {
				const int n = wn * 32 + nt * 8 + gid;
				bfr[nt][0] = ld_pair(&Bs[n][c]);
				bfr[nt][1] = ld_pair(&Bs[n][c + 8]);
			}
#pragma unroll
			for (int mt = 0; mt < 2; mt++)
#pragma unroll
				for (int nt = 0; nt < 4; nt++) {
					float* d = acc[mt][nt];
					asm volatile(
					    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
					    "{%0,%1,%2,%3};\n"
					    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
					    : "r"(af[mt][0]), "r"(af[mt][1]), "r"(af[mt][2]), "r"(af[mt][3]), "r"(bfr[nt][0]),
					      "r"(bfr[nt][1]));
				}
		}
		__syncthreads();
	}
	float* C = g.C ? g.C + z * g.sC : nullptr;
	bf16* Cb = g.Cb ? g.Cb + z * g.sCb : nullptr;
	const float* bias = g.bias ? g.bias + z * g.sBias : nullptr;
#pragma unroll
	for (int mt = 0; mt < 2; mt++)
#pragma unroll
		for (int nt = 0; nt < 4; nt++)
#pragma unroll
			for (int h = 0; h < 2; h++)
#pragma unroll
				for (int q = 0; q < 2; q++) {
					const int m = m0 + wm * 32 + mt * 16 + gid + 8 * h;
					const int n = n0 + wn * 32 + nt * 8 + tig * 2 + q;
					if (m >= g.M || n >= g.N) continue;
					float v = acc[mt][nt][2 * h + q];
					if (bias) v += bias[n];
					if (g.relu) v = fmaxf(v, 0.f);
					if (C) C[(long long)m * g.ldc + n] = v;
					if (Cb) Cb[(long long)m * g.ldcb + n] = __float2bfloat16(v);
				}
}


// The forward product Z = H W^T (A row-major [M][K], B = W row-major [N][K], both
// contiguous in k) as a pipelined kernel: 128x64 output tiles, 8 warps of 32x32,
// K in slices of 32 double-buffered in shared memory by 16-byte cp.async (zero-filled
// past M and K), fragments by ldmatrix, mma.sync m16n8k16 BF16 -> FP32.  Needs K, lda
// and ldb multiples of 8 (the padded widths are multiples of 16).
constexpr int NT_BM = 128, NT_BN = 64, NT_BK = 32, NT_LD = NT_BK + 8;  // 80-byte rows: ldmatrix conflict-free

__device__ __forceinline__ void cp16z(void* smem, const void* gmem, uint32_t bytes) {
	uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(bytes) : "memory");
}
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
	uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
	             : "r"(a));
}

__global__ void __launch_bounds__(256) k_gemm_nt(GemmArgs g) {
	__shared__ __align__(128) bf16 As[2][NT_BM][NT_LD];
	__shared__ __align__(128) bf16 Bs[2][NT_BN][NT_LD];
	const int z = blockIdx.z;
	const bf16* A = g.A + z * g.sA;
	const bf16* B = g.B + z * g.sB;
	const int m0 = blockIdx.y * NT_BM, n0 = blockIdx.x * NT_BN;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int wm = warp >> 1, wn = warp & 1;  // 4 x 2 warps
	const int gid = lane >> 2, tig = lane & 3;
	auto load = [&](int st, int k0) {
		// A: 128 rows x 4 chunks of 8 elements; B: 64 rows x 4 chunks
#pragma unroll
		for (int r = 0; r < 2; r++) {
			const int e = tid + 256 * r, row = e >> 2, ch = e & 3;
			const int m = m0 + row, k = k0 + ch * 8;
			const bool ok = m < g.M && k < g.K;
			cp16z(&As[st][row][ch * 8], ok ? (const void*)(A + (long long)m * g.lda + k) : (const void*)A, ok ? 16u : 0u);
		}
		{
			const int row = tid >> 2, ch = tid & 3;
			const int n = n0 + row, k = k0 + ch * 8;
			const bool ok = n < g.N && k < g.K;
			cp16z(&Bs[st][row][ch * 8], ok ? (const void*)(B + (long long)n * g.ldb + k) : (const void*)B, ok ? 16u : 0u);
		}
		asm volatile("cp.async.commit_group;\n" ::: "memory");
	};
	float acc[2][4][4];
#pragma unroll
	for (int a = 0; a < 2; a++)
#pragma unroll
		for (int b = 0; b < 4; b++)
#pragma unroll
			for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
	const int nk = (g.K + NT_BK - 1) / NT_BK;
	load(0, 0);
	for (int kt = 0; kt < nk; kt++) {
		if (kt + 1 < nk) {
			load((kt + 1) & 1, (kt + 1) * NT_BK);
			asm volatile("cp.async.wait_group 1;\n" ::: "memory");
		} else {
			asm volatile("cp.async.wait_group 0;\n" ::: "memory");
		}
		__syncthreads();
		const int st = kt & 1;
#pragma unroll
		for (int ks = 0; ks < NT_BK; ks += 16) {
			uint32_t af[2][4], bfr[4][2];
#pragma unroll
			for (int mt = 0; mt < 2; mt++) {
				const int r = wm * 32 + mt * 16 + (lane & 15), c = ks + (lane >> 4) * 8;
				ldsm_x4(af[mt][0], af[mt][1], af[mt][2], af[mt][3], &As[st][r][c]);
			}
#pragma unroll
			for (int np = 0; np < 2; np++) {  // two n-tiles of 8 per ldmatrix.x4
				const int r = wn * 32 + np * 16 + (lane & 7) + ((lane >> 4) << 3), c = ks + ((lane >> 3) & 1) * 8;
				ldsm_x4(bfr[2 * np][0], bfr[2 * np][1], bfr[2 * np + 1][0], bfr[2 * np + 1][1], &Bs[st][r][c]);
			}
#pragma unroll
			for (int mt = 0; mt < 2; mt++)
#pragma unroll
				for (int nt = 0; nt < 4; nt++) {
					float* d = acc[mt][nt];
					asm volatile(
					    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
					    "{%0,%1,%2,%3};\n"
					    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
					    : "r"(af[mt][0]), "r"(af[mt][1]), "r"(af[mt][2]), "r"(af[mt][3]), "r"(bfr[nt][0]),
					      "r"(bfr[nt][1]));
				}
		}
		__syncthreads();
	}
	// epilogue: each thread holds column pairs (n, n+1) -- stored as one float2 / bf16x2
	// (N, ldc and ldcb are even: the padded widths are multiples of 16)
	float* C = g.C ? g.C + z * g.sC : nullptr;
	bf16* Cb = g.Cb ? g.Cb + z * g.sCb : nullptr;
	const float* bias = g.bias ? g.bias + z * g.sBias : nullptr;
#pragma unroll
	for (int mt = 0; mt < 2; mt++)
#pragma unroll
		for (int nt = 0; nt < 4; nt++)
#pragma unroll
			for (int h = 0; h < 2; h++) {
				const int m = m0 + wm * 32 + mt * 16 + gid + 8 * h;
				const int n = n0 + wn * 32 + nt * 8 + tig * 2;
				if (m >= g.M || n >= g.N) continue;
				float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
				if (bias) {
					v0 += bias[n];
					v1 += bias[n + 1];
				}
				if (g.relu) {
					v0 = fmaxf(v0, 0.f);
					v1 = fmaxf(v1, 0.f);
				}
				if (C) *reinterpret_cast<float2*>(C + (long long)m * g.ldc + n) = make_float2(v0, v1);
				if (Cb) *reinterpret_cast<__nv_bfloat162*>(Cb + (long long)m * g.ldcb + n) = __floats2bfloat162_rn(v0, v1);
			}
}

// ---- The forward products on Blackwell's tensor cores: tcgen05.mma with the FP32
// accumulators in tensor memory (TMEM), operands staged by TMA.  Z = H W^T for K a
// multiple of 64 and N <= 256 (the 256-wide layers and the output layer).
//
// One persistent CTA per (slice of the row tiles, member); 10 warps with fixed roles:
//   warp 0     one thread issues the TMA copies: the member's whole W once (N x K,
//              K-major, 128-byte swizzled, resident for all of the CTA's tiles), then
//              128-row x 64-column slices of H through a 3-stage ring;
//   warp 1     allocates TMEM (two accumulators of N columns, so that a tile's
//              epilogue overlaps the next tile's products); one thread issues
//              tcgen05.mma (M = 128, N, K = 16, BF16 x BF16 -> FP32) and tcgen05.commit,
//              which releases each H stage and, after a tile's last slice, hands the
//              accumulator to the epilogue;
//   warps 2-9  the epilogue: warp w reads TMEM lanes 32 (w mod 4) .. +31 -- one tile row
//              per thread -- 32 columns at a time (tcgen05.ld; warps 2-5 the even
//              32-column chunks, warps 6-9 the odd ones), adds the bias, applies ReLU
//              and stores FP32 and/or BF16 rows.  Two warps per scheduler in the
//              epilogue hide each other's TMEM-load and store latencies.
// Every mbarrier wait is bounded: past the limit the thread sets the error word and
// leaves its loop; all threads meet at the end, where warp 1 frees the TMEM.
namespace tc {

constexpr int BM = 128;      // tile rows: one TMEM lane each
constexpr int BK = 64;       // K per stage: 64 BF16 = 128 bytes, one 128-byte swizzle span
constexpr int STAGES = 3;
constexpr int EPI = 8;  // epilogue warps: two per TMEM lane quarter, splitting the columns
constexpr int THREADS = 64 + 32 * EPI;
constexpr uint32_t SPIN_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(b)) : "memory");
}
// Wait until the phase of parity `ph` has completed; false after SPIN_LIMIT tries.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t ph) {
	const uint32_t a = saddr(b);
	for (uint32_t it = 0; it < SPIN_LIMIT; it++) {
		uint32_t done;
		asm volatile(
		    "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
		    : "=r"(done)
		    : "r"(a), "r"(ph)
		    : "memory");
		if (done) return true;
	}
	return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
	        saddr(dst)),
	    "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(saddr(bar))
	    : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int x, int y, int z, uint64_t* bar) {
	asm volatile(
	    "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
	        saddr(dst)),
	    "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
	    : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand in the 128-byte-swizzled layout
// that TMA writes: rows of 128 bytes, 8-row groups 1024 bytes apart (stride byte
// offset), descriptor version 1, swizzle mode 2 (128 bytes).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t a) {
	return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
	       ((uint64_t)2 << 61);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
	asm volatile(
	    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
	    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bar))
	             : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// dynamic shared memory: the member's W (K/64 blocks of N rows x 128 B), the H stages
// (128 rows x 128 B each), the mbarriers and the TMEM address; +1 KB for the 1 KB
// alignment that the 128-byte swizzle needs
constexpr int STG_ROW = 144;  // epilogue staging row: 32 FP32 (or 32 BF16) + 16 bytes of padding
__host__ __device__ constexpr size_t smem_bytes(int N, int K) {
	return 1024 + (size_t)(K / BK) * N * 128 + (size_t)STAGES * BM * 128 + EPI * 32 * STG_ROW + 8 * (1 + 2 * STAGES + 4) + 16;
}
__host__ __device__ constexpr uint32_t tmem_cols(int N) { return N <= 128 ? 256u : 512u; }

__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW, GemmArgs g,
              int rows_per_member, uint32_t* err) {
	extern __shared__ uint8_t smem_raw[];
	const int N = g.N, KB = g.K / BK, G = gridDim.x, z = blockIdx.y;
	const uint32_t raw = saddr(smem_raw);
	uint8_t* sW = smem_raw + (((raw + 1023u) & ~1023u) - raw);
	uint8_t* sA = sW + (size_t)KB * N * 128;
	uint8_t* sStg = sA + (size_t)STAGES * BM * 128;  // EPI epilogue warps x 32 rows x STG_ROW
	uint64_t* w_full = reinterpret_cast<uint64_t*>(sStg + EPI * 32 * STG_ROW);
	uint64_t* a_full = w_full + 1;
	uint64_t* a_empty = a_full + STAGES;
	uint64_t* acc_full = a_empty + STAGES;
	uint64_t* acc_empty = acc_full + 2;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int tiles = (g.M + BM - 1) / BM;
	const uint32_t ncols = tmem_cols(N), acc_stride = ncols / 2;

	if (threadIdx.x == 0) {
		mbar_init(w_full, 1);
		for (int s = 0; s < STAGES; s++) {
			mbar_init(a_full + s, 1);
			mbar_init(a_empty + s, 1);
		}
		for (int b = 0; b < 2; b++) {
			mbar_init(acc_full + b, 1);
			mbar_init(acc_empty + b, EPI);  // one arrival per epilogue warp
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tmem_slot)),
		             "r"(ncols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	fence_before();
	__syncthreads();
	fence_after();
	const uint32_t tmem = *tmem_slot;
	bool ok = true;

	if (warp == 0) {
		if (lane == 0) {  // TMA producer
			mbar_expect_tx(w_full, (uint32_t)(KB * N * 128));
			for (int kb = 0; kb < KB; kb++) tma_load_3d(sW + (size_t)kb * N * 128, &tmW, kb * BK, 0, z, w_full);
			uint32_t it = 0;
			for (int t = blockIdx.x; t < tiles && ok; t += G)
				for (int kb = 0; kb < KB; kb++, it++) {
					const int s = (int)(it % STAGES);
					const uint32_t use = it / STAGES;
					if (use > 0 && !(ok = mbar_wait(a_empty + s, (use - 1) & 1u))) break;
					mbar_expect_tx(a_full + s, BM * 128);
					tma_load_2d(sA + (size_t)s * BM * 128, &tmA, kb * BK, z * rows_per_member + t * BM, a_full + s);
				}
		}
	} else if (warp == 1) {
		if (lane == 0) {  // MMA issuer
			const uint32_t idesc = idesc_bf16(BM, N);
			ok = mbar_wait(w_full, 0);
			uint32_t it = 0, i = 0;
			for (int t = blockIdx.x; t < tiles && ok; t += G, i++) {
				const uint32_t ab = i & 1u, use = i >> 1;
				if (use > 0 && !(ok = mbar_wait(acc_empty + ab, (use - 1) & 1u))) break;
				fence_after();
				const uint32_t d = tmem + ab * acc_stride;
				for (int kb = 0; kb < KB; kb++, it++) {
					const int s = (int)(it % STAGES);
					if (!(ok = mbar_wait(a_full + s, (it / STAGES) & 1u))) break;
					fence_after();
					const uint32_t a0 = saddr(sA + (size_t)s * BM * 128), b0 = saddr(sW + (size_t)kb * N * 128);
#pragma unroll
					for (int k = 0; k < BK / 16; k++)  // K = 16 per instruction: 32 bytes along the swizzled row
						mma_bf16(d, sw128_desc(a0 + 32u * k), sw128_desc(b0 + 32u * k), idesc, (kb | k) != 0);
					mma_commit(a_empty + s);  // the stage is free once these products are done
				}
				if (ok) mma_commit(acc_full + ab);
			}
		}
	} else {  // epilogue
		// each warp stages its 32 rows x 32 columns in shared memory (rows padded to
		// 144 bytes: the 16-byte accesses of 8 lanes hit distinct banks) and writes
		// them out coalesced -- BF16: 16-byte chunks, 8 rows of 64 bytes per
		// instruction; FP32: one row of up to 128 bytes per instruction, any ldc
		const int q = warp & 3, grp = (warp - 2) >> 2;  // lane quarter; column group (chunks grp, grp + 2, ...)
		uint8_t* stg = sStg + (size_t)(warp - 2) * 32 * STG_ROW;
		const float* bias = g.bias ? g.bias + z * g.sBias : nullptr;
		float* C = g.C ? g.C + z * g.sC : nullptr;
		bf16* Cb = g.Cb ? g.Cb + z * g.sCb : nullptr;
		const int nst = g.n_store > 0 ? g.n_store : N;
		uint32_t i = 0;
		for (int t = blockIdx.x; t < tiles && ok; t += G, i++) {
			const uint32_t ab = i & 1u;
			if (!(ok = mbar_wait(acc_full + ab, (i >> 1) & 1u))) break;
			fence_after();
			const int row0 = t * BM + 32 * q;  // this warp's first row
			const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + ab * acc_stride;
			for (int c0 = 32 * grp; c0 < N; c0 += 64) {
				uint32_t r[32];
				tmem_ld32(taddr + (uint32_t)c0, r);  // row 32q + lane, columns c0..c0+31
				float v[32];
#pragma unroll
				for (int j = 0; j < 32; j++) {
					float x = __uint_as_float(r[j]);
					if (bias && c0 + j < N) x += bias[c0 + j];
					if (g.relu) x = fmaxf(x, 0.f);
					v[j] = x;
				}
				if (Cb) {
					uint4* srow = reinterpret_cast<uint4*>(stg + lane * STG_ROW);
#pragma unroll
					for (int j = 0; j < 4; j++) {
						__nv_bfloat162 h0 = __floats2bfloat162_rn(v[8 * j], v[8 * j + 1]);
						__nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 * j + 2], v[8 * j + 3]);
						__nv_bfloat162 h2 = __floats2bfloat162_rn(v[8 * j + 4], v[8 * j + 5]);
						__nv_bfloat162 h3 = __floats2bfloat162_rn(v[8 * j + 6], v[8 * j + 7]);
						srow[j] = make_uint4(*reinterpret_cast<uint32_t*>(&h0), *reinterpret_cast<uint32_t*>(&h1),
						                     *reinterpret_cast<uint32_t*>(&h2), *reinterpret_cast<uint32_t*>(&h3));
					}
					__syncwarp();
#pragma unroll
					for (int k = 0; k < 4; k++) {
						const int e = lane + 32 * k, rr = e >> 2, ch = e & 3, m = row0 + rr;
						if (m < g.M && c0 + 8 * ch < N)
							*reinterpret_cast<uint4*>(Cb + (long long)m * g.ldcb + c0 + 8 * ch) =
							    *reinterpret_cast<const uint4*>(stg + rr * STG_ROW + 16 * ch);
					}
					__syncwarp();
				}
				if (C) {
					float4* srow = reinterpret_cast<float4*>(stg + lane * STG_ROW);
#pragma unroll
					for (int j = 0; j < 8; j++) srow[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
					__syncwarp();
					if (c0 + lane < nst)
						for (int rr = 0; rr < 32; rr++) {
							const int m = row0 + rr;
							if (m < g.M) C[(long long)m * g.ldc + c0 + lane] = reinterpret_cast<const float*>(stg + rr * STG_ROW)[lane];
						}
					__syncwarp();
				}
			}
			fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(acc_empty + ab);
		}
	}
	if (!ok) atomicOr(err, 1u);
	fence_before();
	__syncthreads();
	fence_after();
	if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(ncols) : "memory");
}

}  // namespace tc

// Fused inference: the whole forward pass of every member in one persistent kernel,
// the hidden activations never leaving the SM.  A CTA takes tiles of 256 rows of one
// member (two halves of 128 rows, one TMEM accumulator of up to 256 FP32 columns each)
// and runs them through all layers:
//   - the epilogue warps write the tile's input rows (FP32 -> BF16, zero padded to the
//     first layer's K) into shared memory in the 128-byte-swizzled K-major layout that
//     a TMA load would produce, so the tensor core reads them as an operand: per 64-wide
//     K chunk the 256 rows in order (half 0's 128, then half 1's);
//   - the producer (warp 0) streams each layer's BF16 weights, 64-wide K chunks of all
//     N rows, through a ring of shared-memory stages with TMA;
//   - the MMA issuer (warp 1) multiplies, per K chunk, both halves (A = the half's rows,
//     B = the weights: M = 128, N = the layer's width) and commits each half's
//     accumulator after its last chunk.  An M = 128 product takes about as long for any
//     N up to 256, so the narrow output layer runs transposed: A = its weights (the
//     outputs padded to 128 or 256 rows by the tensor map's zero fill), B = all 256 rows
//     of the tile (N = 256), half the products of two M = 128 halves;
//   - the epilogue warps (8: four TMEM lane quarters x two halves) read their half's
//     accumulator (two TMEM loads in flight: the next 32 columns load while these are
//     converted), add the bias, apply ReLU, round to BF16 and write the next layer's
//     operand over the current one (whose products are complete by then); after the
//     output layer a warp holds 32 consecutive outputs (TMEM lanes) of its half's rows
//     (columns), adds the bias and stores each row's 32 outputs with one coalesced store.
// Only the inputs (in FP32), the weights (from L2: every CTA on a member reads the same
// ones) and the outputs move through memory.  The products are the per-layer path's --
// BF16 operands, FP32 accumulation in K order, the bias added in FP32 -- with K padded
// to 64 by zeros.  Every wait is bounded; on a timeout the kernel sets the error word,
// waits (bounded) for its own copies and products in flight, frees the TMEM and returns.
namespace fz {

constexpr int TILE = 256, HALF = 128;
constexpr int CHUNK = HALF * 128;  // one 64-wide K chunk of a half: 128 rows x 128 bytes
constexpr int EPI = 8;
constexpr int THREADS = 64 + 32 * EPI;
constexpr uint32_t TMEM_COLS = 512;  // two accumulators of up to 256 columns

struct Maps {
	CUtensorMap w[MF_MLP_MAX_LAYERS];  // per layer: [members][N][K] BF16, boxes of 64 K x N rows
};
struct Args {
	int L, in, out, rows, stages, kc_max, n_max;
	int N[MF_MLP_MAX_LAYERS], KC[MF_MLP_MAX_LAYERS];  // MMA width (padded to 16); K / 64 (K padded to 64)
	int mb_last;                                       // 128-row blocks of the transposed output layer (1 or 2)
	int b_off[MF_MLP_MAX_LAYERS];
	const float* bias;
	long long b_per;
	const float* x;  // x[z * sx + r * in + c] (sx = 0: one input shared by the members)
	long long sx;
	float* y;  // y[z * sy + r * ldy + c]
	long long sy;
	int ldy;
	int members;
};

// the mbarriers (2 per weight stage, 2 x 2 per half, 1 to drain) and the TMEM address,
// rounded up to 16 bytes
__host__ __device__ constexpr size_t bar_bytes(int stages) { return (8 * (2 * stages + 5) + 4 + 15) / 16 * 16; }
// shared memory: 1 KB for the 1 KB alignment of the swizzled operands, the operand
// chunks of the tile, the weight stages, the barriers and one layer's bias
__host__ __device__ constexpr size_t smem_bytes(int kc_max, int n_max, int stages) {
	return 1024 + (size_t)2 * kc_max * CHUNK + (size_t)stages * n_max * 128 + bar_bytes(stages) + (size_t)n_max * 4;
}

// the 16-byte unit holding columns col .. col + 7 (col a multiple of 8) of row r of half
// h: K chunk col / 64 (the chunk's 256 rows: half 0, then half 1), unit (col % 64) / 8
// XOR (r % 8) -- the 128-byte swizzle
__device__ __forceinline__ uint4* unit_at(uint8_t* act, int h, int r, int col) {
	const int kc = col >> 6, u = (col >> 3) & 7;
	return reinterpret_cast<uint4*>(act + (size_t)(2 * kc + h) * CHUNK + r * 128 + ((u ^ (r & 7)) << 4));
}
__device__ __forceinline__ uint32_t pack2(float a, float b) {
	__nv_bfloat162 h = __floats2bfloat162_rn(a, b);
	return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// max(a, 0) and max(b, 0) rounded to BF16, a in the low half
__device__ __forceinline__ uint32_t pack2_relu(float a, float b) {
	uint32_t d;
	asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(b), "f"(a));
	return d;
}
// 32 columns of the warp's 32 TMEM lanes without waiting (tmem_wait before use)
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t* r) {
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// named barrier 1 over the 256 epilogue threads; epi_all also returns the AND of p over them
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 256;\n" ::: "memory"); }
__device__ __forceinline__ bool epi_all(bool p) {
	uint32_t r;
	asm volatile("{\n.reg .pred q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred q, 1, 256, q;\nselp.u32 %0, 1, 0, q;\n}\n"
	             : "=r"(r)
	             : "r"((uint32_t)p)
	             : "memory");
	return r != 0;
}

// 32 accumulator columns col0 .. col0 + 31 of row r (in v) -> bias (sb4: the layer's bias
// in shared memory), ReLU, BF16 -> their four 16-byte units of the next operand; columns
// at or past N (the layer's width) become zeros up to the next layer's K
__device__ __forceinline__ void hidden_units(uint8_t* act, int h, int r, int col0, int N, const uint32_t* v,
                                             const float4* sb4) {
#pragma unroll
	for (int u = 0; u < 4; u++) {
		const int col = col0 + 8 * u;
		uint4 w = make_uint4(0, 0, 0, 0);
		if (col < N) {
			const float4 b0 = sb4[col >> 2], b1 = sb4[(col >> 2) + 1];
			float f[8];
#pragma unroll
			for (int e = 0; e < 8; e++) f[e] = __uint_as_float(v[8 * u + e]);
			w = make_uint4(pack2_relu(f[0] + b0.x, f[1] + b0.y), pack2_relu(f[2] + b0.z, f[3] + b0.w),
			               pack2_relu(f[4] + b1.x, f[5] + b1.y), pack2_relu(f[6] + b1.z, f[7] + b1.w));
		}
		*unit_at(act, h, r, col) = w;
	}
}

__global__ void __launch_bounds__(THREADS, 1)
    k_mlp_fused(const __grid_constant__ Maps maps, const Args a, uint32_t* err) {
	using namespace tc;
	extern __shared__ uint8_t smem_raw[];
	const uint32_t raw = saddr(smem_raw);
	uint8_t* act = smem_raw + (((raw + 1023u) & ~1023u) - raw);
	const size_t wst = (size_t)a.n_max * 128;
	const int S = a.stages, L = a.L;
	uint8_t* sW = act + (size_t)2 * a.kc_max * CHUNK;
	uint64_t* w_full = reinterpret_cast<uint64_t*>(sW + (size_t)S * wst);
	uint64_t* w_empty = w_full + S;
	uint64_t* acc_full = w_empty + S;    // per half: the layer's products are complete
	uint64_t* act_ready = acc_full + 2;  // per half: the operand of the next layer is written
	uint64_t* fin = act_ready + 2;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);
	float* sbias = reinterpret_cast<float*>(sW + (size_t)S * wst + bar_bytes(S));  // the current layer's bias
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int tpm = (a.rows + TILE - 1) / TILE, total = tpm * a.members;

	if (threadIdx.x == 0) {
		for (int s = 0; s < S; s++) {
			mbar_init(w_full + s, 1);
			mbar_init(w_empty + s, 1);
		}
		for (int h = 0; h < 2; h++) {
			mbar_init(acc_full + h, 1);
			mbar_init(act_ready + h, 32 * EPI / 2);  // every thread of the half's four warps
		}
		mbar_init(fin, 1);
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tmem_slot)),
		             "r"(TMEM_COLS)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	fence_before();
	__syncthreads();
	fence_after();
	const uint32_t tmem = *tmem_slot;
	bool ok = true;

	if (warp == 0) {
		if (lane == 0) {  // weight producer
			uint32_t it = 0;
			for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
				const int z = t % a.members;
				for (int l = 0; l < L && ok; l++) {
					// the output layer's box is 128 * mb_last rows, zero filled past its width
					const uint32_t bytes = (uint32_t)(l + 1 < L ? a.N[l] : 128 * a.mb_last) * 128u;
					for (int kc = 0; kc < a.KC[l]; kc++, it++) {
						const int s = (int)(it % S);
						const uint32_t use = it / S;
						if (use > 0 && !(ok = mbar_wait(w_empty + s, (use - 1) & 1u))) break;
						mbar_expect_tx(w_full + s, bytes);
						tma_load_3d(sW + (size_t)s * wst, &maps.w[l], kc * 64, 0, z, w_full + s);
					}
				}
			}
			// the loads still in flight land before the CTA leaves (consumed ones: at once)
			for (uint32_t k = it > (uint32_t)S ? it - S : 0; k < it; k++) mbar_wait(w_full + k % S, (k / S) & 1u);
		}
	} else if (warp == 1) {
		if (lane == 0) {  // MMA issuer
			uint32_t it = 0, step = 0;
			bool issued = false;
			for (int t = blockIdx.x; t < total && ok; t += gridDim.x)
				for (int l = 0; l < L && ok; l++, step++) {
					if (!(ok = mbar_wait(act_ready, step & 1u)) || !(ok = mbar_wait(act_ready + 1, step & 1u))) break;
					fence_after();
					const bool last = l + 1 == L;
					const uint32_t idesc = last ? idesc_bf16(HALF, TILE) : idesc_bf16(HALF, a.N[l]);
					for (int kc = 0; kc < a.KC[l]; kc++, it++) {
						const int s = (int)(it % S);
						if (!(ok = mbar_wait(w_full + s, (it / S) & 1u))) break;
						fence_after();
						const uint32_t wb = saddr(sW + (size_t)s * wst), ab = saddr(act + (size_t)2 * kc * CHUNK);
						if (!last) {
							for (int h = 0; h < 2; h++) {  // D[row][n] of half h: A = its rows, B = the weights
								const uint32_t a0 = ab + (uint32_t)(h * CHUNK);
#pragma unroll
								for (int k = 0; k < 4; k++)  // K = 16 per instruction: 32 bytes along the swizzled row
									mma_bf16(tmem + (uint32_t)(h * 256), sw128_desc(a0 + 32u * k), sw128_desc(wb + 32u * k), idesc,
									         (kc | k) != 0);
								if (kc == a.KC[l] - 1) mma_commit(acc_full + h);
							}
						} else {
							for (int mb = 0; mb < a.mb_last; mb++) {  // D[out][row]: A = 128 weight rows, B = the tile's 256 rows
								const uint32_t w0 = wb + (uint32_t)(mb * CHUNK);
#pragma unroll
								for (int k = 0; k < 4; k++)
									mma_bf16(tmem + (uint32_t)(mb * 256), sw128_desc(w0 + 32u * k), sw128_desc(ab + 32u * k), idesc,
									         (kc | k) != 0);
							}
							if (kc == a.KC[l] - 1) {
								mma_commit(acc_full);
								mma_commit(acc_full + 1);
							}
						}
						mma_commit(w_empty + s);  // the stage is free once these products are done
						issued = true;
					}
				}
			if (issued) {  // nothing of this CTA's left in the tensor pipe before the TMEM is freed
				mma_commit(fin);
				mbar_wait(fin, 0);
			}
		}
	} else {  // epilogue: half h, TMEM lane quarter q, row r of the half
		const int h = (warp - 2) >> 2, q = warp & 3, r = 32 * q + lane, et = threadIdx.x - 64;
		const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);  // this warp's lane quarter
		const float4* sb4 = reinterpret_cast<const float4*>(sbias);
		// tile tt: member tt % members (CTAs running side by side read different members'
		// weights), rows (tt / members) * 256 + ...; the first 8 input columns of this
		// thread's row are fetched ahead into registers
		float xp[8];
		auto x_fetch = [&](int tt) {
			const int grow = (tt / a.members) * TILE + h * HALF + r;
			const bool live = grow < a.rows;
			const float* xr = a.x + (tt % a.members) * a.sx + (long long)(live ? grow : 0) * a.in;
#pragma unroll
			for (int j = 0; j < 8; j++) xp[j] = live && j < a.in ? xr[j] : 0.f;
		};
		auto x_write = [&](int tt) {  // the input row, BF16, zero padded to the first layer's K
			*unit_at(act, h, r, 0) = make_uint4(pack2(xp[0], xp[1]), pack2(xp[2], xp[3]), pack2(xp[4], xp[5]), pack2(xp[6], xp[7]));
			const int grow = (tt / a.members) * TILE + h * HALF + r;
			const bool live = grow < a.rows;
			const float* xr = a.x + (tt % a.members) * a.sx + (long long)(live ? grow : 0) * a.in;
			for (int col = 8; col < a.KC[0] * 64; col += 8) {
				float f[8];
#pragma unroll
				for (int j = 0; j < 8; j++) f[j] = live && col + j < a.in ? xr[col + j] : 0.f;
				*unit_at(act, h, r, col) = make_uint4(pack2(f[0], f[1]), pack2(f[2], f[3]), pack2(f[4], f[5]), pack2(f[6], f[7]));
			}
			proxy_fence();  // generic-proxy writes, read next by the tensor core
			mbar_arrive(act_ready + h);
		};
		// the bias of layer l of tile tt's member into shared memory (all 256 threads)
		auto fill = [&](int tt, int l) {
			const float* src = a.bias + (tt % a.members) * a.b_per + a.b_off[l];
			for (int i = et; i < a.N[l]; i += 32 * EPI) sbias[i] = src[i];
		};
		int t = blockIdx.x;
		if (t < total) {
			x_fetch(t);
			fill(t, 0);
		}
		epi_sync();
		if (t < total) x_write(t);
		uint32_t step = 0;
		for (; t < total && ok; t += gridDim.x) {
			const int z = t % a.members, row0 = (t / a.members) * TILE + h * HALF, tn = t + gridDim.x;
			for (int l = 0; l < L; l++, step++) {
				const bool last = l + 1 == L;
				if (last && tn < total) x_fetch(tn);  // its latency hides under the products
				const bool mine = mbar_wait(acc_full + h, step & 1u);
				if (mine) {
					fence_after();
					const int N = a.N[l];
					uint32_t va[32], vb[32];
					if (!last) {
						// this half's accumulator, 32 columns at a time, the next 32 loading
						// while these are converted
						const uint32_t acc = tq + (uint32_t)(h * 256);
						const int Kn = 64 * a.KC[l + 1];
						if (N > 0) tmem_ld32_async(acc, va);
						tmem_wait();
						for (int c0 = 0; c0 < Kn; c0 += 64) {
							if (c0 + 32 < N) tmem_ld32_async(acc + (uint32_t)(c0 + 32), vb);
							hidden_units(act, h, r, c0, N, va, sb4);
							tmem_wait();
							if (c0 + 64 < N) tmem_ld32_async(acc + (uint32_t)(c0 + 64), va);
							hidden_units(act, h, r, c0 + 32, N, vb, sb4);
							tmem_wait();
						}
						fence_before();
						proxy_fence();
						mbar_arrive(act_ready + h);
					} else {
						// D[output f][tile row]: this warp holds outputs 128 mb + 32 q + lane of
						// its half's 128 rows (columns 128 h ..); one coalesced store per row
						float* yz = a.y + z * a.sy;
						for (int mb = 0; mb < a.mb_last; mb++) {
							if (128 * mb + 32 * q >= a.out) continue;  // no output of this warp here
							const int f = 128 * mb + 32 * q + lane;
							const float bf = f < N ? sbias[f] : 0.f;
							const bool fo = f < a.out;
							const uint32_t acc = tq + (uint32_t)(mb * 256 + h * HALF);
							tmem_ld32_async(acc, va);
							tmem_wait();
							for (int p = 0; p < 4; p += 2) {
								tmem_ld32_async(acc + (uint32_t)(32 * (p + 1)), vb);
#pragma unroll
								for (int j = 0; j < 32; j++) {
									const int gr = row0 + 32 * p + j;
									if (fo && gr < a.rows) yz[(long long)gr * a.ldy + f] = __uint_as_float(va[j]) + bf;
								}
								tmem_wait();
								if (p + 2 < 4) tmem_ld32_async(acc + (uint32_t)(32 * (p + 2)), va);
#pragma unroll
								for (int j = 0; j < 32; j++) {
									const int gr = row0 + 32 * (p + 1) + j;
									if (fo && gr < a.rows) yz[(long long)gr * a.ldy + f] = __uint_as_float(vb[j]) + bf;
								}
								tmem_wait();
							}
						}
						fence_before();
						if (tn < total) x_write(tn);
					}
				}
				// every epilogue thread is done with this step's bias, and all agree on
				// going on (a wait that gave up ends the loop for all 256 together)
				ok = epi_all(mine);
				if (!ok) break;
				if (!last) fill(t, l + 1);
				else if (tn < total) fill(tn, 0);
				epi_sync();
			}
		}
	}
	if (!ok) atomicOr(err, 1u);
	fence_before();
	__syncthreads();
	fence_after();
	if (warp == 1)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// weights of one layer for the fused kernel: [members][N][Kp] BF16, K padded to Kp
// (a multiple of 64) by zeros
__global__ void k_pack_layer(int members, int N, int K, int Kp, const bf16* src, long long s_per, bf16* dst,
                             long long d_per) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	const long long per = (long long)N * Kp;
	if (e >= per * members) return;
	const int z = (int)(e / per);
	const long long w = e % per;
	const int o = (int)(w / Kp), i = (int)(w % Kp);
	dst[z * d_per + w] = i < K ? src[z * s_per + (long long)o * K + i] : __float2bfloat16(0.f);
}

}  // namespace fz

// Training control block in device memory, read by the graph's kernels on every replay.
struct TrainCtl {
	uint32_t step;   // Adam steps taken so far (the current step's number inside a step)
	uint32_t t0;     // step count when the current mf_mlp_train call began
	uint32_t total;  // steps of the current call (cosine schedule length)
	uint32_t n_data;
	float lr0, lr1;
	float* hist;  // [total][members] loss history of the current call
	uint64_t seed;
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}

// bootstrap minibatch: member z's row r takes data row splitmix(seed, step, z, r) mod n
__global__ void k_gather(const TrainCtl* ctl, int in, int in_p, int out, long long sH0, long long sY, const float* X,
                         const float* Y, bf16* H0, float* Yb) {
	const int r = blockIdx.x, z = blockIdx.y;
	const uint64_t key = ctl->seed ^ ((uint64_t)ctl->step << 20) ^ ((uint64_t)z << 52) ^ (uint64_t)r;
	const uint32_t src = (uint32_t)(splitmix64(key) % ctl->n_data);
	for (int c = threadIdx.x; c < in_p; c += blockDim.x)
		H0[z * sH0 + (long long)r * in_p + c] = __float2bfloat16(c < in ? X[(long long)src * in + c] : 0.f);
	for (int c = threadIdx.x; c < out; c += blockDim.x) Yb[z * sY + (long long)r * out + c] = Y[(long long)src * out + c];
}

// x (FP32 [batch][in] per member, member stride sx; 0 = shared) -> BF16 [batch][in_p], zero padded
__global__ void k_input(int members, int batch, int in, int in_p, const float* x, long long sx, bf16* h, long long sh) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	const long long per = (long long)batch * in_p;
	if (e >= per * members) return;
	const int z = (int)(e / per);
	const long long w = e % per;
	const int c = (int)(w % in_p);
	const long long r = w / in_p;
	h[z * sh + w] = __float2bfloat16(c < in ? x[z * sx + r * in + c] : 0.f);
}

// mean squared error of member z over batch x out; dZ = 2 (y_pred - y) / (batch * out)
__global__ void k_mse(int batch, int out, int out_p, const float* yp, long long syp, const float* y, long long sy,
                      float* dz, bf16* dzb, long long sdz, float* loss) {
	const int z = blockIdx.y;
	float s = 0.f;
	const float inv = 1.f / (float)(batch * out);
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < batch * out_p; e += gridDim.x * blockDim.x) {
		const int c = e % out_p, r = e / out_p;
		float d = 0.f;
		if (c < out) {
			const float diff = yp[z * syp + e] - y[z * sy + (long long)r * out + c];
			s += diff * diff;
			d = 2.f * diff * inv;
		}
		dz[z * sdz + e] = d;
		dzb[z * sdz + e] = __float2bfloat16(d);
	}
	__shared__ float red[256];
	red[threadIdx.x] = s;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) atomicAdd(&loss[z], red[0] * inv);
}

// dZ = dH where the layer's ReLU output H > 0, else 0 (FP32 and BF16 copies)
__global__ void k_relu_bwd(int members, long long per, const float* dh, long long sdh, const bf16* h, long long sh,
                           float* dz, bf16* dzb, long long sdz) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= per * members) return;
	const int z = (int)(e / per);
	const long long w = e % per;
	const float v = __bfloat162float(h[z * sh + w]) > 0.f ? dh[z * sdh + w] : 0.f;
	dz[z * sdz + w] = v;
	dzb[z * sdz + w] = __float2bfloat16(v);
}

// db[n] = sum over rows of dZ[r][n]
__global__ void k_bias_grad(int batch, int out_p, const float* dz, long long sdz, float* db, long long sdb) {
	const int n = blockIdx.x * blockDim.x + threadIdx.x, z = blockIdx.y;
	if (n >= out_p) return;
	const float* d = dz + z * sdz;
	float s = 0.f;
	for (int r = 0; r < batch; r++) s += d[(long long)r * out_p + n];
	db[z * sdb + n] = s;
}

// Adam (Kingma & Ba 2015) on FP32 master parameters with a cosine learning-rate
// schedule from lr0 to lr1 over the current call; refreshes the BF16 weight copy.
__global__ void k_adam(const TrainCtl* ctl, long long n, float* w, const float* g, float* m, float* v, bf16* wb) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n) return;
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	const uint32_t t = ctl->step;
	const float frac = ctl->total > 1 ? (float)(t - 1 - ctl->t0) / (float)(ctl->total - 1) : 0.f;
	const float lr = ctl->lr1 + 0.5f * (ctl->lr0 - ctl->lr1) * (1.f + cospif(fminf(fmaxf(frac, 0.f), 1.f)));
	const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
	const float gi = g[e];
	const float mi = b1 * m[e] + (1.f - b1) * gi;
	const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
	m[e] = mi;
	v[e] = vi;
	const float wi = w[e] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	w[e] = wi;
	if (wb) wb[e] = __float2bfloat16(wi);
}

__global__ void k_step_begin(TrainCtl* ctl, float* loss, int members) {
	if (threadIdx.x == 0) ctl->step += 1;
	for (int z = threadIdx.x; z < members; z += blockDim.x) loss[z] = 0.f;
}

__global__ void k_step_end(const TrainCtl* ctl, const float* loss, int members) {
	const uint32_t row = ctl->step - 1 - ctl->t0;
	if (!ctl->hist || row >= ctl->total) return;
	for (int z = threadIdx.x; z < members; z += blockDim.x) ctl->hist[(size_t)row * members + z] = loss[z];
}

__global__ void k_to_bf16(long long n, const float* a, bf16* b) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (e < n) b[e] = __float2bfloat16(a[e]);
}

// unpadded outputs [members][rows][out] from the padded last layer [members][rows][out_p]
__global__ void k_output(int members, int rows, int out, int out_p, const float* yp, long long syp, float* y,
                         long long sy) {
	const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	const long long per = (long long)rows * out;
	if (e >= per * members) return;
	const int z = (int)(e / per);
	const long long w = e % per;
	y[z * sy + w] = yp[z * syp + (w / out) * out_p + (w % out)];
}

inline int pad16(int v) { return (v + 15) / 16 * 16; }
inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <class T>
struct Buf {
	T* p = nullptr;
	size_t n = 0;
	cudaError_t alloc(size_t count) {
		free();
		n = count;
		return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
	}
	void free() {
		if (p) cudaFree(p);
		p = nullptr;
		n = 0;
	}
	~Buf() { free(); }
};

// portable seeded initialisation: splitmix64 -> uniform in [-1, 1)
struct HostRng {
	uint64_t s;
	uint64_t next() {
		uint64_t x = (s += 0x9E3779B97F4A7C15ull);
		x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
		x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
		return x ^ (x >> 31);
	}
	float sym() { return (float)((double)(next() >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0); }
};

}  // namespace

struct mf_mlp {
	int members = 0, L = 0, rows = 0, device = 0;
	std::vector<int> dims, pd;            // true and padded widths, L + 1 each
	std::vector<long long> w_off, b_off;  // per-layer offsets inside one member's block
	long long w_per = 0, b_per = 0;       // parameters per member (padded)
	int widest = 0;
	Buf<float> W, Bias, gW, gB, mW, vW, mB, vB;
	Buf<bf16> Wb;
	std::vector<Buf<bf16>> H;  // H[l]: BF16 [members][rows][pd[l]], l = 0..L-1
	Buf<float> Yp;             // FP32 [members][rows][pd[L]]
	Buf<float> dz, dh;         // FP32 [members][rows][widest]
	Buf<bf16> dzb;
	Buf<float> loss;           // [members]
	Buf<float> Xin, Yin;       // batches from the host: [members][rows][in], [members][rows][out]
	Buf<float> Xd, Yd;         // training set [n][in], [n][out]
	Buf<float> hist;
	Buf<TrainCtl> ctl;
	TrainCtl h_ctl{};
	cudaStream_t stream = nullptr;
	cudaGraphExec_t graph = nullptr;
	uint64_t launches = 0, step_launches = 0;
	std::string err;
	bool tc = false;       // forward products with K % 64 == 0 on tcgen05 (else mma.sync)
	bool fused = true;     // with tc: inference through the fused whole-network kernel when it applies
	int sm_count = 1;
	// fused inference: the BF16 weights re-laid per layer as [members][N][K padded to 64],
	// their tensor maps, and the kernel's shared-memory plan
	Buf<bf16> Wf;
	std::vector<long long> wf_off;
	long long wf_per = 0;
	bool wf_dirty = true;  // Wb changed since Wf was packed
	fz::Maps maps{};
	int fz_kc = 1, fz_n = 16, fz_stages = 0;
	Buf<uint32_t> dev_err; // set by a bounded wait of the tcgen05 GEMM that gave up
	~mf_mlp() {
		if (graph) cudaGraphExecDestroy(graph);
		if (stream) cudaStreamDestroy(stream);
	}
};

namespace {

mf_status mlp_fail(mf_mlp* m, const std::string& what, cudaError_t e) {
	m->err = what + ": " + cudaGetErrorString(e);
	return MF_ERR_CUDA;
}
#define MCK(call)                                             \
	do {                                                      \
		cudaError_t e_ = (call);                              \
		if (e_ != cudaSuccess) return mlp_fail(m, #call, e_); \
	} while (0)

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda)
EncodeTiled tensor_map_encoder() {
	static EncodeTiled fn = [] {
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q{};
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
		    q != cudaDriverEntryPointSuccess)
			p = nullptr;
		return reinterpret_cast<EncodeTiled>(p);
	}();
	return fn;
}

constexpr size_t TC_SMEM_MAX = 227 * 1024;

// The tcgen05 path takes the forward products Z = H W^T whose operands are contiguous
// K-major rows with K a multiple of 64, N a multiple of 16 up to 256, and whose staged
// operands fit the shared memory; H is [members][rows][K], W [N][K] per member.
bool tc_eligible(const mf_mlp* m, bool ta, bool tb, const GemmArgs& g) {
	return m->tc && !ta && tb && g.K % tc::BK == 0 && g.N % 16 == 0 && g.N <= 256 && g.lda == g.K && g.ldb == g.K &&
	       g.sA == (long long)m->rows * g.K && g.M <= m->rows && tc::smem_bytes(g.N, g.K) <= TC_SMEM_MAX &&
	       (!g.Cb || g.ldcb % 8 == 0) && g.sB % 8 == 0;
}

cudaError_t gemm_tc(mf_mlp* m, const GemmArgs& g) {
	EncodeTiled enc = tensor_map_encoder();
	CUtensorMap tA, tW;
	// H as [members * rows][K]; boxes of 64 K x 128 rows, 128-byte swizzle, zero fill past the end
	const cuuint64_t dA[2] = {(cuuint64_t)g.K, (cuuint64_t)m->members * m->rows};
	const cuuint64_t sA[1] = {(cuuint64_t)g.K * 2};
	const cuuint32_t bA[2] = {tc::BK, tc::BM}, e1[3] = {1, 1, 1};
	// W as [members][N][K] (member stride sB elements); boxes of 64 K x N rows x 1 member
	const cuuint64_t dW[3] = {(cuuint64_t)g.K, (cuuint64_t)g.N, (cuuint64_t)m->members};
	const cuuint64_t sW[2] = {(cuuint64_t)g.K * 2, (cuuint64_t)g.sB * 2};
	const cuuint32_t bW[3] = {tc::BK, (cuuint32_t)g.N, 1};
	if (enc(&tA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(g.A), dA, sA, bA, e1,
	        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
	    enc(&tW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(g.B), dW, sW, bW, e1,
	        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
		return cudaErrorInvalidValue;
	const int tiles = (g.M + tc::BM - 1) / tc::BM;
	const int G = std::max(1, std::min(tiles, m->sm_count / m->members));
	tc::k_gemm_tc<<<dim3(G, m->members), tc::THREADS, tc::smem_bytes(g.N, g.K), m->stream>>>(tA, tW, g, m->rows,
	                                                                                         m->dev_err.p);
	m->launches++;
	return cudaGetLastError();
}

cudaError_t gemm(mf_mlp* m, bool ta, bool tb, GemmArgs g) {
	dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM, m->members);
	cudaStream_t s = m->stream;
	if (tc_eligible(m, ta, tb, g)) return gemm_tc(m, g);
	if (!ta && tb && g.K % 8 == 0 && g.lda % 8 == 0 && g.ldb % 8 == 0 && g.N % 2 == 0 && (!g.C || g.ldc % 2 == 0) &&
	    (!g.Cb || g.ldcb % 2 == 0)) {
		dim3 gnt((g.N + NT_BN - 1) / NT_BN, (g.M + NT_BM - 1) / NT_BM, m->members);
		k_gemm_nt<<<gnt, 256, 0, s>>>(g);
	} else if (!ta && tb) k_gemm<false, true><<<grid, 128, 0, s>>>(g);
	else if (!ta && !tb) k_gemm<false, false><<<grid, 128, 0, s>>>(g);
	else if (ta && !tb) k_gemm<true, false><<<grid, 128, 0, s>>>(g);
	else k_gemm<true, true><<<grid, 128, 0, s>>>(g);
	m->launches++;
	return cudaGetLastError();
}

long long sH(const mf_mlp* m, int l) { return (long long)m->rows * m->pd[l]; }

// The fused inference kernel takes models whose padded widths are all at most 256 (one
// accumulator per half tile, at most four K chunks) and whose operands leave room for at
// least two weight stages in shared memory.
void fused_plan(mf_mlp* m) {
	m->fz_kc = 1;
	m->fz_n = 16;
	bool fits = true;
	for (int l = 0; l < m->L; l++) {
		m->fz_kc = std::max(m->fz_kc, (m->pd[l] + 63) / 64);
		// the output layer's weight box: 128 or 256 rows (it runs transposed, M = 128 per block)
		m->fz_n = std::max(m->fz_n, l + 1 < m->L ? m->pd[l + 1] : (m->pd[l + 1] + 127) / 128 * 128);
		fits = fits && m->pd[l] <= 256 && m->pd[l + 1] <= 256;
	}
	m->fz_stages = 0;
	if (fits)
		for (int st = 4; st >= 2 && !m->fz_stages; st--)
			if (fz::smem_bytes(m->fz_kc, m->fz_n, st) <= TC_SMEM_MAX) m->fz_stages = st;
}

bool fused_eligible(const mf_mlp* m) { return m->tc && m->fused && m->fz_stages >= 2; }

// (re)packs the BF16 weights for the fused kernel and encodes one tensor map per layer:
// [members][N][Kp] with member stride wf_per, boxes of 64 K x N rows x 1 member
mf_status fused_prepare(mf_mlp* m) {
	if (!m->wf_dirty) return MF_OK;
	if (!m->Wf.p) {
		m->wf_off.clear();
		m->wf_per = 0;
		for (int l = 0; l < m->L; l++) {
			m->wf_off.push_back(m->wf_per);
			m->wf_per += (long long)m->pd[l + 1] * ((m->pd[l] + 63) / 64 * 64);
		}
		MCK(m->Wf.alloc((size_t)m->wf_per * m->members));
	}
	EncodeTiled enc = tensor_map_encoder();
	for (int l = 0; l < m->L; l++) {
		const int N = m->pd[l + 1], K = m->pd[l], Kp = (K + 63) / 64 * 64;
		const long long per = (long long)N * Kp * m->members;
		fz::k_pack_layer<<<nblk(per, 256), 256, 0, m->stream>>>(m->members, N, K, Kp, m->Wb.p + m->w_off[l], m->w_per,
		                                                      m->Wf.p + m->wf_off[l], m->wf_per);
		m->launches++;
		MCK(cudaGetLastError());
		const cuuint64_t dW[3] = {(cuuint64_t)Kp, (cuuint64_t)N, (cuuint64_t)m->members};
		const cuuint64_t sW[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)m->wf_per * 2};
		const cuuint32_t box_rows = l + 1 < m->L ? (cuuint32_t)N : (cuuint32_t)((N + 127) / 128 * 128);  // zero filled past N
		const cuuint32_t bW[3] = {64, box_rows, 1}, e1[3] = {1, 1, 1};
		if (enc(&m->maps.w[l], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, m->Wf.p + m->wf_off[l], dW, sW, bW, e1,
		        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
		        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
			m->err = "fused inference: encoding a weight tensor map failed";
			return MF_ERR_CUDA;
		}
	}
	m->wf_dirty = false;
	return MF_OK;
}

// all members over `rows` rows: x[z * sx + r * in + c] -> y[z * sy + r * ldy + c]
cudaError_t fused_forward(mf_mlp* m, const float* x, long long sx, int rows, float* y, long long sy, int ldy) {
	if (rows <= 0) return cudaSuccess;
	fz::Args a{};
	a.L = m->L;
	a.in = m->dims[0];
	a.out = m->dims[m->L];
	a.rows = rows;
	a.stages = m->fz_stages;
	a.kc_max = m->fz_kc;
	a.n_max = m->fz_n;
	a.mb_last = (m->pd[m->L] + 127) / 128;
	for (int l = 0; l < m->L; l++) {
		a.N[l] = m->pd[l + 1];
		a.KC[l] = (m->pd[l] + 63) / 64;
		a.b_off[l] = (int)m->b_off[l];
	}
	a.bias = m->Bias.p;
	a.b_per = m->b_per;
	a.x = x;
	a.sx = sx;
	a.y = y;
	a.sy = sy;
	a.ldy = ldy;
	a.members = m->members;
	const long long tiles = (long long)(rows + fz::TILE - 1) / fz::TILE * m->members;
	const int G = (int)std::min<long long>(tiles, m->sm_count);
	fz::k_mlp_fused<<<G, fz::THREADS, fz::smem_bytes(a.kc_max, a.n_max, a.stages), m->stream>>>(m->maps, a,
	                                                                                           m->dev_err.p);
	m->launches++;
	return cudaGetLastError();
}

bool device_pointer(const void* p) {
	cudaPointerAttributes at{};
	if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// forward pass of all members over `batch` rows already in H[0]
// direct_out: when the last layer runs on tcgen05, write its unpadded outputs straight
// into Yin ([members][rows][out], FP32) and set *wrote_direct (no unpadding pass then)
cudaError_t forward_layers(mf_mlp* m, int batch, bool direct_out = false, bool* wrote_direct = nullptr) {
	if (wrote_direct) *wrote_direct = false;
	for (int l = 0; l < m->L; l++) {
		GemmArgs g{};
		g.M = batch; g.N = m->pd[l + 1]; g.K = m->pd[l];
		g.A = m->H[l].p; g.lda = m->pd[l]; g.sA = sH(m, l);
		g.B = m->Wb.p + m->w_off[l]; g.ldb = m->pd[l]; g.sB = m->w_per;
		g.bias = m->Bias.p + m->b_off[l]; g.sBias = m->b_per;
		if (l + 1 < m->L) {
			g.Cb = m->H[l + 1].p; g.ldcb = m->pd[l + 1]; g.sCb = sH(m, l + 1);
			g.relu = 1;
		} else {
			g.C = m->Yp.p; g.ldc = m->pd[l + 1]; g.sC = sH(m, l + 1);
			if (direct_out && tc_eligible(m, false, true, g)) {
				g.C = m->Yin.p; g.ldc = m->dims[m->L]; g.sC = (long long)m->rows * m->dims[m->L];
				g.n_store = m->dims[m->L];
				if (wrote_direct) *wrote_direct = true;
			}
		}
		cudaError_t e = gemm(m, false, true, g);
		if (e != cudaSuccess) return e;
	}
	return cudaSuccess;
}

// gradients of the mean squared error against y (FP32 [members][rows][out]) into gW,
// gB; the per-member losses accumulate into m->loss (zeroed beforehand)
cudaError_t backward_layers(mf_mlp* m, const float* y, int batch) {
	cudaStream_t s = m->stream;
	const int L = m->L;
	const long long sdz = (long long)m->rows * m->widest;  // member stride of dz, dh, dzb
	k_mse<<<dim3(32, m->members), 256, 0, s>>>(batch, m->dims[L], m->pd[L], m->Yp.p, sH(m, L), y,
	                                           (long long)m->rows * m->dims[L], m->dz.p, m->dzb.p, sdz, m->loss.p);
	m->launches++;
	for (int l = L - 1; l >= 0; l--) {
		const int out_p = m->pd[l + 1], in_p = m->pd[l];
		k_bias_grad<<<dim3(nblk(out_p, 128), m->members), 128, 0, s>>>(batch, out_p, m->dz.p, sdz, m->gB.p + m->b_off[l],
		                                                               m->b_per);
		m->launches++;
		// dW [out x in] = dZ^T [out x batch] . H[l] [batch x in]
		GemmArgs gw{};
		gw.M = out_p; gw.N = in_p; gw.K = batch;
		gw.A = m->dzb.p; gw.lda = out_p; gw.sA = sdz;
		gw.B = m->H[l].p; gw.ldb = in_p; gw.sB = sH(m, l);
		gw.C = m->gW.p + m->w_off[l]; gw.ldc = in_p; gw.sC = m->w_per;
		cudaError_t e = gemm(m, true, false, gw);
		if (e != cudaSuccess) return e;
		if (l == 0) break;
		// dH [batch x in] = dZ [batch x out] . W [out x in]
		GemmArgs gx{};
		gx.M = batch; gx.N = in_p; gx.K = out_p;
		gx.A = m->dzb.p; gx.lda = out_p; gx.sA = sdz;
		gx.B = m->Wb.p + m->w_off[l]; gx.ldb = in_p; gx.sB = m->w_per;
		gx.C = m->dh.p; gx.ldc = in_p; gx.sC = sdz;
		if ((e = gemm(m, false, false, gx)) != cudaSuccess) return e;
		const long long per = (long long)batch * in_p;
		k_relu_bwd<<<nblk(per * m->members, 256), 256, 0, s>>>(m->members, per, m->dh.p, sdz, m->H[l].p, sH(m, l), m->dz.p,
		                                                      m->dzb.p, sdz);
		m->launches++;
	}
	return cudaGetLastError();
}

cudaError_t adam_update(mf_mlp* m) {
	const long long nw = m->w_per * m->members, nb = m->b_per * m->members;
	k_adam<<<nblk(nw, 256), 256, 0, m->stream>>>(m->ctl.p, nw, m->W.p, m->gW.p, m->mW.p, m->vW.p, m->Wb.p);
	k_adam<<<nblk(nb, 256), 256, 0, m->stream>>>(m->ctl.p, nb, m->Bias.p, m->gB.p, m->mB.p, m->vB.p, nullptr);
	m->launches += 2;
	return cudaGetLastError();
}

// one full training step on the stream (this sequence is what the graph captures)
cudaError_t train_step_launches(mf_mlp* m) {
	cudaStream_t s = m->stream;
	const int out = m->dims[m->L];
	k_step_begin<<<1, 64, 0, s>>>(m->ctl.p, m->loss.p, m->members);
	k_gather<<<dim3(m->rows, m->members), 32, 0, s>>>(m->ctl.p, m->dims[0], m->pd[0], out, sH(m, 0),
	                                                  (long long)m->rows * out, m->Xd.p, m->Yd.p, m->H[0].p, m->Yin.p);
	m->launches += 2;
	cudaError_t e;
	if ((e = forward_layers(m, m->rows)) != cudaSuccess) return e;
	if ((e = backward_layers(m, m->Yin.p, m->rows)) != cudaSuccess) return e;
	if ((e = adam_update(m)) != cudaSuccess) return e;
	k_step_end<<<1, 64, 0, s>>>(m->ctl.p, m->loss.p, m->members);
	m->launches++;
	return cudaGetLastError();
}

// MF_ERR_TIMEOUT (and the error word cleared) when a tcgen05 GEMM gave up a wait
mf_status tc_status(mf_mlp* m) {
	if (!m->tc) return MF_OK;
	uint32_t e = 0;
	MCK(cudaMemcpy(&e, m->dev_err.p, 4, cudaMemcpyDeviceToHost));
	if (!e) return MF_OK;
	MCK(cudaMemset(m->dev_err.p, 0, 4));
	m->err = "tcgen05 GEMM: a bounded wait gave up";
	return MF_ERR_TIMEOUT;
}

void drop_graph(mf_mlp* m) {
	if (m->graph) cudaGraphExecDestroy(m->graph);
	m->graph = nullptr;
}

// parameters of one member, unpadded, layer by layer: W_l [out][in] row-major, then b_l
enum class Walk { GetParams, GetGrads, SetParams };
mf_status param_walk(mf_mlp* m, int member, float* host, Walk mode) {
	size_t o = 0;
	float* Wsrc = mode == Walk::GetGrads ? m->gW.p : m->W.p;
	float* Bsrc = mode == Walk::GetGrads ? m->gB.p : m->Bias.p;
	const bool get = mode != Walk::SetParams;
	for (int l = 0; l < m->L; l++) {
		const size_t wdev = (size_t)member * m->w_per + m->w_off[l];
		const size_t wid = (size_t)m->dims[l] * 4, pitch = (size_t)m->pd[l] * 4;
		if (get) MCK(cudaMemcpy2D(host + o, wid, Wsrc + wdev, pitch, wid, m->dims[l + 1], cudaMemcpyDeviceToHost));
		else MCK(cudaMemcpy2D(Wsrc + wdev, pitch, host + o, wid, wid, m->dims[l + 1], cudaMemcpyHostToDevice));
		o += (size_t)m->dims[l] * m->dims[l + 1];
		const size_t bdev = (size_t)member * m->b_per + m->b_off[l];
		if (get) MCK(cudaMemcpy(host + o, Bsrc + bdev, m->dims[l + 1] * 4, cudaMemcpyDeviceToHost));
		else MCK(cudaMemcpy(Bsrc + bdev, host + o, m->dims[l + 1] * 4, cudaMemcpyHostToDevice));
		o += m->dims[l + 1];
	}
	return MF_OK;
}

}  // namespace

extern "C" {

MF_API mf_status mf_mlp_create(const mf_mlp_config* cfg, mf_mlp** out) {
	if (!cfg || !out) return MF_ERR_ARG;
	*out = nullptr;
	if (cfg->members < 1 || cfg->members > 64 || cfg->n_layers < 1 || cfg->n_layers > MF_MLP_MAX_LAYERS ||
	    cfg->max_batch < 1)
		return MF_ERR_ARG;
	if (cfg->max_batch > 65535) return MF_ERR_CAPACITY;  // gridDim.y of the GEMM tiles and the gather
	for (int l = 0; l <= cfg->n_layers; l++) {
		if (cfg->dims[l] < 1) return MF_ERR_ARG;
		if (cfg->dims[l] > MF_MLP_MAX_WIDTH) return MF_ERR_CAPACITY;
	}
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MF_ERR_NO_DEVICE;
	if (cfg->device < 0 || cfg->device >= ndev) return MF_ERR_ARG;
	if (cudaSetDevice(cfg->device) != cudaSuccess) return MF_ERR_NO_DEVICE;
	mf_mlp* m = new mf_mlp();
	m->members = cfg->members;
	m->L = cfg->n_layers;
	m->rows = cfg->max_batch;
	m->device = cfg->device;
	for (int l = 0; l <= m->L; l++) {
		m->dims.push_back(cfg->dims[l]);
		m->pd.push_back(pad16(cfg->dims[l]));
		m->widest = std::max(m->widest, m->pd.back());
	}
	for (int l = 0; l < m->L; l++) {
		m->w_off.push_back(m->w_per);
		m->b_off.push_back(m->b_per);
		m->w_per += (long long)m->pd[l + 1] * m->pd[l];
		m->b_per += m->pd[l + 1];
	}
	const long long nw = m->w_per * m->members, nb = m->b_per * m->members;
	// He-uniform weights U(-sqrt(6/fan_in), sqrt(6/fan_in)), zero biases, zero padding
	std::vector<float> hw(nw, 0.f);
	HostRng rng{cfg->seed};
	for (int z = 0; z < m->members; z++)
		for (int l = 0; l < m->L; l++) {
			const float lim = std::sqrt(6.f / (float)m->dims[l]);
			for (int o = 0; o < m->dims[l + 1]; o++)
				for (int i = 0; i < m->dims[l]; i++)
					hw[z * m->w_per + m->w_off[l] + (long long)o * m->pd[l] + i] = lim * rng.sym();
		}
	auto setup = [&]() -> mf_status {
		MCK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
		Buf<float>* wbufs[] = {&m->W, &m->gW, &m->mW, &m->vW};
		for (auto* b : wbufs) {
			MCK(b->alloc(nw));
			MCK(cudaMemset(b->p, 0, nw * 4));
		}
		Buf<float>* bbufs[] = {&m->Bias, &m->gB, &m->mB, &m->vB};
		for (auto* b : bbufs) {
			MCK(b->alloc(nb));
			MCK(cudaMemset(b->p, 0, nb * 4));
		}
		MCK(m->Wb.alloc(nw));
		MCK(cudaMemcpy(m->W.p, hw.data(), nw * 4, cudaMemcpyHostToDevice));
		k_to_bf16<<<nblk(nw, 256), 256, 0, m->stream>>>(nw, m->W.p, m->Wb.p);
		m->launches++;
		MCK(cudaGetLastError());
		m->H.resize(m->L);
		for (int l = 0; l < m->L; l++) MCK(m->H[l].alloc((size_t)m->members * sH(m, l)));
		const size_t act = (size_t)m->members * m->rows * m->widest;
		MCK(m->Yp.alloc((size_t)m->members * sH(m, m->L)));
		MCK(m->dz.alloc(act));
		MCK(m->dh.alloc(act));
		MCK(m->dzb.alloc(act));
		MCK(m->loss.alloc(m->members));
		MCK(m->Xin.alloc((size_t)m->members * m->rows * m->dims[0]));
		MCK(m->Yin.alloc((size_t)m->members * m->rows * m->dims[m->L]));
		MCK(m->ctl.alloc(1));
		MCK(m->dev_err.alloc(1));
		MCK(cudaMemset(m->dev_err.p, 0, 4));
		// the tcgen05 forward products on Blackwell (compute capability 10.x), where the
		// driver provides the tensor-map encoder
		int major = 0;
		MCK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, m->device));
		MCK(cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device));
		m->tc = major == 10 && tensor_map_encoder() != nullptr;
		fused_plan(m);
		if (m->tc) {
			MCK(cudaFuncSetAttribute(tc::k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_MAX));
			MCK(cudaFuncSetAttribute(fz::k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_MAX));
		}
		m->h_ctl = TrainCtl{};
		m->h_ctl.seed = cfg->seed * 0x2545F4914F6CDD1Dull + 1;
		MCK(cudaMemcpy(m->ctl.p, &m->h_ctl, sizeof(TrainCtl), cudaMemcpyHostToDevice));
		MCK(cudaStreamSynchronize(m->stream));
		return MF_OK;
	};
	mf_status st = setup();
	if (st != MF_OK) {
		delete m;
		return st;
	}
	*out = m;
	return MF_OK;
}

MF_API void mf_mlp_destroy(mf_mlp* m) {
	if (!m) return;
	cudaSetDevice(m->device);
	delete m;
}

MF_API const char* mf_mlp_last_error(const mf_mlp* m) { return m ? m->err.c_str() : "null model"; }

MF_API mf_status mf_mlp_num_params(const mf_mlp* m, uint64_t* n) {
	if (!m || !n) return MF_ERR_ARG;
	uint64_t t = 0;
	for (int l = 0; l < m->L; l++) t += (uint64_t)m->dims[l + 1] * m->dims[l] + m->dims[l + 1];
	*n = t;
	return MF_OK;
}

MF_API mf_status mf_mlp_get_params(mf_mlp* m, int32_t member, float* host) {
	if (!m || !host || member < 0 || member >= m->members) return MF_ERR_ARG;
	MCK(cudaSetDevice(m->device));
	MCK(cudaStreamSynchronize(m->stream));
	return param_walk(m, member, host, Walk::GetParams);
}

MF_API mf_status mf_mlp_get_grads(mf_mlp* m, int32_t member, float* host) {
	if (!m || !host || member < 0 || member >= m->members) return MF_ERR_ARG;
	MCK(cudaSetDevice(m->device));
	MCK(cudaStreamSynchronize(m->stream));
	return param_walk(m, member, host, Walk::GetGrads);
}

MF_API mf_status mf_mlp_set_params(mf_mlp* m, int32_t member, const float* host) {
	if (!m || !host || member < 0 || member >= m->members) return MF_ERR_ARG;
	MCK(cudaSetDevice(m->device));
	MCK(cudaStreamSynchronize(m->stream));
	mf_status st = param_walk(m, member, const_cast<float*>(host), Walk::SetParams);
	if (st != MF_OK) return st;
	const long long nw = m->w_per * m->members;
	k_to_bf16<<<nblk(nw, 256), 256, 0, m->stream>>>(nw, m->W.p, m->Wb.p);
	m->launches++;
	m->wf_dirty = true;
	MCK(cudaGetLastError());
	MCK(cudaStreamSynchronize(m->stream));
	return MF_OK;
}

MF_API mf_status mf_mlp_gradients(mf_mlp* m, const float* x, const float* y, int32_t batch, float* loss) {
	if (!m || !x || !y || batch < 1) return MF_ERR_ARG;
	if (batch > m->rows) return MF_ERR_CAPACITY;
	MCK(cudaSetDevice(m->device));
	cudaStream_t s = m->stream;
	const int in = m->dims[0], out = m->dims[m->L];
	// [members][batch][...] rows into the [members][rows][...] slots
	MCK(cudaMemcpy2DAsync(m->Xin.p, (size_t)m->rows * in * 4, x, (size_t)batch * in * 4, (size_t)batch * in * 4,
	                      m->members, cudaMemcpyDefault, s));
	MCK(cudaMemcpy2DAsync(m->Yin.p, (size_t)m->rows * out * 4, y, (size_t)batch * out * 4, (size_t)batch * out * 4,
	                      m->members, cudaMemcpyDefault, s));
	MCK(cudaMemsetAsync(m->loss.p, 0, m->members * 4, s));
	const long long per = (long long)batch * m->pd[0];
	k_input<<<nblk(per * m->members, 256), 256, 0, s>>>(m->members, batch, in, m->pd[0], m->Xin.p,
	                                                    (long long)m->rows * in, m->H[0].p, sH(m, 0));
	m->launches++;
	MCK(cudaGetLastError());
	MCK(forward_layers(m, batch));
	MCK(backward_layers(m, m->Yin.p, batch));
	if (loss) MCK(cudaMemcpyAsync(loss, m->loss.p, m->members * 4, cudaMemcpyDefault, s));
	MCK(cudaStreamSynchronize(s));
	return MF_OK;
}

MF_API mf_status mf_mlp_set_data(mf_mlp* m, const float* x, const float* y, int32_t n) {
	if (!m || !x || !y || n < 1) return MF_ERR_ARG;
	MCK(cudaSetDevice(m->device));
	MCK(cudaStreamSynchronize(m->stream));
	const int in = m->dims[0], out = m->dims[m->L];
	if (m->Xd.n < (size_t)n * in || m->Yd.n < (size_t)n * out) {
		drop_graph(m);  // the captured gather holds the data pointers
		MCK(m->Xd.alloc((size_t)n * in));
		MCK(m->Yd.alloc((size_t)n * out));
	}
	MCK(cudaMemcpy(m->Xd.p, x, (size_t)n * in * 4, cudaMemcpyDefault));
	MCK(cudaMemcpy(m->Yd.p, y, (size_t)n * out * 4, cudaMemcpyDefault));
	m->h_ctl.n_data = (uint32_t)n;
	return MF_OK;
}

MF_API mf_status mf_mlp_train(mf_mlp* m, int32_t steps, float lr0, float lr1, float* loss_history) {
	if (!m || steps < 0 || !(lr0 >= 0.f) || !(lr1 >= 0.f)) return MF_ERR_ARG;
	if (!m->h_ctl.n_data) {
		m->err = "mf_mlp_train: no training data (call mf_mlp_set_data first)";
		return MF_ERR_STATE;
	}
	if (!steps) return MF_OK;
	MCK(cudaSetDevice(m->device));
	cudaStream_t s = m->stream;
	MCK(cudaStreamSynchronize(s));
	if (m->hist.n < (size_t)steps * m->members) MCK(m->hist.alloc((size_t)steps * m->members));
	// the device step counter is authoritative; rewrite the schedule fields around it
	TrainCtl cur;
	MCK(cudaMemcpy(&cur, m->ctl.p, sizeof(TrainCtl), cudaMemcpyDeviceToHost));
	m->h_ctl.step = cur.step;
	m->h_ctl.t0 = cur.step;
	m->h_ctl.total = (uint32_t)steps;
	m->h_ctl.lr0 = lr0;
	m->h_ctl.lr1 = lr1;
	m->h_ctl.hist = m->hist.p;
	MCK(cudaMemcpy(m->ctl.p, &m->h_ctl, sizeof(TrainCtl), cudaMemcpyHostToDevice));
	if (!m->graph) {
		cudaGraph_t g = nullptr;
		MCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		const uint64_t before = m->launches;
		cudaError_t e = train_step_launches(m);
		cudaError_t e2 = cudaStreamEndCapture(s, &g);
		m->step_launches = m->launches - before;
		m->launches = before;
		if (e != cudaSuccess || e2 != cudaSuccess) {
			if (g) cudaGraphDestroy(g);
			return mlp_fail(m, "capturing the training step", e != cudaSuccess ? e : e2);
		}
		e = cudaGraphInstantiate(&m->graph, g, 0);
		cudaGraphDestroy(g);
		if (e != cudaSuccess) {
			m->graph = nullptr;
			return mlp_fail(m, "cudaGraphInstantiate", e);
		}
	}
	m->wf_dirty = true;
	for (int t = 0; t < steps; t++) MCK(cudaGraphLaunch(m->graph, s));
	m->launches += m->step_launches * (uint64_t)steps;
	if (loss_history)
		MCK(cudaMemcpyAsync(loss_history, m->hist.p, (size_t)steps * m->members * 4, cudaMemcpyDefault, s));
	MCK(cudaStreamSynchronize(s));
	return tc_status(m);
}

MF_API mf_status mf_mlp_predict(mf_mlp* m, const float* x, int32_t n, float* y) {
	if (!m || n < 0 || (n > 0 && (!x || !y))) return MF_ERR_ARG;
	MCK(cudaSetDevice(m->device));
	cudaStream_t s = m->stream;
	const int in = m->dims[0], out = m->dims[m->L];
	if (n > 0 && fused_eligible(m)) {
		mf_status st = fused_prepare(m);
		if (st != MF_OK) return st;
		const bool xd = device_pointer(x), yd = device_pointer(y);
		if (xd && yd) {  // one launch over every row, straight from x into y
			MCK(fused_forward(m, x, 0, n, y, (long long)n * out, out));
		} else
			for (int r0 = 0; r0 < n; r0 += m->rows) {
				const int b = std::min(m->rows, n - r0);
				const float* xs = x + (size_t)r0 * in;
				if (!xd) {
					MCK(cudaMemcpyAsync(m->Xin.p, xs, (size_t)b * in * 4, cudaMemcpyDefault, s));
					xs = m->Xin.p;
				}
				if (yd) {
					MCK(fused_forward(m, xs, 0, b, y + (size_t)r0 * out, (long long)n * out, out));
				} else {
					MCK(fused_forward(m, xs, 0, b, m->Yin.p, (long long)m->rows * out, out));
					MCK(cudaMemcpy2DAsync(y + (size_t)r0 * out, (size_t)n * out * 4, m->Yin.p, (size_t)m->rows * out * 4,
					                      (size_t)b * out * 4, m->members, cudaMemcpyDefault, s));
				}
			}
		MCK(cudaStreamSynchronize(s));
		return tc_status(m);
	}
	for (int r0 = 0; r0 < n; r0 += m->rows) {
		const int b = std::min(m->rows, n - r0);
		MCK(cudaMemcpyAsync(m->Xin.p, x + (size_t)r0 * in, (size_t)b * in * 4, cudaMemcpyDefault, s));
		const long long per = (long long)b * m->pd[0];
		k_input<<<nblk(per * m->members, 256), 256, 0, s>>>(m->members, b, in, m->pd[0], m->Xin.p, 0, m->H[0].p, sH(m, 0));
		m->launches++;
		MCK(cudaGetLastError());
		bool direct = false;
		MCK(forward_layers(m, b, true, &direct));
		// unpadded outputs into Yin ([members][rows][out]) -- written there by the last
		// layer itself on the tcgen05 path -- then one 2D copy per chunk
		if (!direct) {
			const long long po = (long long)b * out;
			k_output<<<nblk(po * m->members, 256), 256, 0, s>>>(m->members, b, out, m->pd[m->L], m->Yp.p, sH(m, m->L),
			                                                   m->Yin.p, (long long)m->rows * out);
			m->launches++;
			MCK(cudaGetLastError());
		}
		MCK(cudaMemcpy2DAsync(y + (size_t)r0 * out, (size_t)n * out * 4, m->Yin.p, (size_t)m->rows * out * 4,
		                      (size_t)b * out * 4, m->members, cudaMemcpyDefault, s));
	}
	MCK(cudaStreamSynchronize(s));
	return tc_status(m);
}

MF_API mf_status mf_mlp_launch_count(const mf_mlp* m, uint64_t* launches) {
	if (!m || !launches) return MF_ERR_ARG;
	*launches = m->launches;
	return MF_OK;
}

MF_API mf_status mf_mlp_get_stream(const mf_mlp* m, void** stream) {
	if (!m || !stream) return MF_ERR_ARG;
	*stream = (void*)m->stream;
	return MF_OK;
}

MF_API mf_status mf_mlp_set_option(mf_mlp* m, const char* key, int64_t value) {
	if (!m || !key) return MF_ERR_ARG;
	if (!strcmp(key, "tcgen05")) {
		if (value != 0 && value != 1) return MF_ERR_ARG;
		int major = 0;
		MCK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, m->device));
		if (value && !(major == 10 && tensor_map_encoder())) {
			m->err = "tcgen05: needs a compute capability 10.x device and the driver's tensor-map encoder";
			return MF_ERR_STATE;
		}
		if (value && !m->tc) {
			MCK(cudaFuncSetAttribute(tc::k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_MAX));
			MCK(cudaFuncSetAttribute(fz::k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_MAX));
		}
		m->tc = value != 0;
		drop_graph(m);  // the captured training step holds the old launches
		return MF_OK;
	}
	if (!strcmp(key, "fused")) {
		if (value != 0 && value != 1) return MF_ERR_ARG;
		m->fused = value != 0;
		return MF_OK;
	}
	m->err = std::string("unknown option ") + key;
	return MF_ERR_ARG;
}

MF_API mf_status mf_mlp_get_option(const mf_mlp* m, const char* key, int64_t* value) {
	if (!m || !key || !value) return MF_ERR_ARG;
	if (!strcmp(key, "tcgen05")) {
		*value = m->tc ? 1 : 0;
		return MF_OK;
	}
	if (!strcmp(key, "fused")) {  // 1 when predict runs the fused kernel
		*value = fused_eligible(m) ? 1 : 0;
		return MF_OK;
	}
	return MF_ERR_ARG;
}

}  // extern "C"
