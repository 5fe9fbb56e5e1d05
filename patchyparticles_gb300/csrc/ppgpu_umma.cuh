/*
 * ppgpu_umma.cuh -- fifth-generation tensor-core (tcgen05) building blocks for the learned proposal's
 * per-particle MLP, written as inline PTX for sm_103a. Header-only: included by the colour kernels
 * (inference inside the learned move) and by ppgpu_mlp.cu (standalone forward, training step).
 *
 * Operands live in shared memory in the canonical no-swizzle K-major layout: a matrix of R rows and K
 * columns (bf16) is a grid of 8 x 8 core matrices, each 128 contiguous bytes (8 rows of 16 bytes), the
 * core matrices of one 8-row group stored one after the other along K. In the shared-memory descriptor
 * the leading-dimension byte offset (core matrices adjacent in K) is therefore 128 and the
 * stride-dimension byte offset (adjacent 8-row groups) is K / 8 * 128. One tcgen05.mma (kind::f16,
 * cta_group::1) computes D[128 x N] (+)= A[128 x 16] . B[N x 16]^T with D in tensor memory, FP32; a
 * K = 16 step advances both descriptors' start address by two core matrices (256 bytes).
 *
 * Row i of a 128-row D is tensor-memory lane i, column j is column base + j; warp w of the CTA reads
 * lanes 32 (w % 4) .. 32 (w % 4) + 31 (tcgen05.ld .32x32b), so with 128 threads thread t owns row t.
 *
 * Every wait on an mbarrier has an iteration limit: on expiry the caller gets false, records an error
 * and still releases its tensor memory.
 */
#ifndef PPGPU_UMMA_CUH_
#define PPGPU_UMMA_CUH_

#include <cuda_bf16.h>
#include <stddef.h>
#include <stdint.h>

/* ---------------------------------------------------------------- network shape (fixed) */
#define MLP_IN 36      /* 3 neighbours x 4 patch sites x 3 components */
#define MLP_K1 48      /* layer-1 K padded to a multiple of 16 */
#define MLP_HID 64
#define MLP_OUT 4      /* mixture logits */
#define MLP_N3 16      /* layer-3 N padded to the smallest legal N for M = 128 */
#define MLP_ROWS 128   /* particles per tensor-core tile */
#define MLP_SAMPLE 40  /* floats per training sample: 36 features, 4 component utilities */

/* FP32 master parameters, the layout the C-ABI exposes: W1[64][36] b1[64] W2[64][64] b2[64] W3[4][64] b3[4] */
#define MLP_OFF_W1 0
#define MLP_OFF_B1 (MLP_OFF_W1 + MLP_HID * MLP_IN)
#define MLP_OFF_W2 (MLP_OFF_B1 + MLP_HID)
#define MLP_OFF_B2 (MLP_OFF_W2 + MLP_HID * MLP_HID)
#define MLP_OFF_W3 (MLP_OFF_B2 + MLP_HID)
#define MLP_OFF_B3 (MLP_OFF_W3 + MLP_OUT * MLP_HID)
#define MLP_NPARAMS (MLP_OFF_B3 + MLP_OUT)

/* packed BF16 operand image in global memory (bytes), copied verbatim into shared memory:
 *   W1 [64 x 48]  layer-1 B operand (columns 36..47 zero)
 *   W2 [64 x 64]  layer-2 B operand
 *   W3 [16 x 64]  layer-3 B operand (rows 4..15 zero)
 *   W3T[64 x 16]  B operand of dH2 = dZ . W3 (columns 4..15 zero)
 *   W2T[64 x 64]  B operand of dH1 = dA2 . W2
 *   bias: b1[64] b2[64] b3[4] as FP32 (+ padding) */
#define MLPI_W1 0
#define MLPI_W2 (MLPI_W1 + MLP_HID * MLP_K1 * 2)
#define MLPI_W3 (MLPI_W2 + MLP_HID * MLP_HID * 2)
#define MLPI_W3T (MLPI_W3 + MLP_N3 * MLP_HID * 2)
#define MLPI_W2T (MLPI_W3T + MLP_HID * MLP_N3 * 2)
#define MLPI_BIAS (MLPI_W2T + MLP_HID * MLP_HID * 2)
#define MLPI_FWD_BYTES (MLPI_W3T) /* the forward pass needs W1, W2, W3 */
#define MLPI_BYTES (MLPI_BIAS + (2 * MLP_HID + 16) * 4)

/* element offset of (r, k) in a canonical K-major matrix with K columns */
__host__ __device__ __forceinline__ int cl_off(int r, int k, int K) { return ((((r >> 3) * (K >> 3)) + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7); }

/* instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
 * K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28 */
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

/* shared-memory matrix descriptor, no swizzle: start >> 4 (bits 0-13), leading-dimension byte offset
 * >> 4 (16-29), stride-dimension byte offset >> 4 (32-45), descriptor version 1 (bits 46-48 = 0b001),
 * base offset 0, layout type 0 (bits 61-63) */
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
	return (uint64_t) ((saddr >> 4) & 0x3FFFu) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* descriptor of a canonical K-major matrix with K columns starting at smem address saddr */
__device__ __forceinline__ uint64_t umma_kmajor(uint32_t saddr, int K) { return umma_sdesc(saddr, 128u, (uint32_t) (K >> 3) * 128u); }

/* ---------------------------------------------------------------- tensor memory */
/* executed by one whole warp (converged first: .sync.aligned); the allocated base address is written to
 * *dst (shared memory) */
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
	__syncwarp();
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
	__syncwarp();
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* generic-proxy shared-memory writes made visible to the tensor core's (async proxy) reads */
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* ---------------------------------------------------------------- mbarrier */
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
	uint32_t ok;
	asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok)
			: "r"(smem_u32(bar)), "r"(parity)
			: "memory");
	return ok != 0u;
}

#define UMMA_WAIT_CYCLES (1ll << 31) /* ~1 s at the SM clock: a wait that long has failed */

/* wait for the phase with the given parity to complete; false when the time limit (SM clock cycles)
 * expired. Lanes may leave the loop in different rounds: callers reconverge before any .sync.aligned
 * instruction. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = UMMA_WAIT_CYCLES) {
	const long long t0 = clock64();
	while(!mbar_try_wait(bar, parity))
		if(clock64() - t0 > limit) return false;
	return true;
}

/* one arrival on *bar from the calling thread */
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}

/* ---------------------------------------------------------------- MMA issue (one thread) */
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
	asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"setp.ne.b32 p, %4, 0;\n\t"
			"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
			"l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
			: "memory");
}

/* completion of every MMA this thread issued so far arrives once on *bar */
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

/* D[128 x N] = A[128 x K] . B[N x K]^T, both canonical K-major in shared memory, D at tensor-memory
 * column address d_tmem; issued by one thread, K / 16 instructions */
__device__ __forceinline__ void umma_gemm(uint32_t d_tmem, const void *A, const void *B, int K, int N) {
	const uint32_t a = smem_u32(A), b = smem_u32(B);
	const uint32_t idesc = umma_idesc_bf16(128, N);
	for(int k = 0; k < K / 16; k++) umma_bf16(d_tmem, umma_kmajor(a + 256u * k, K), umma_kmajor(b + 256u * k, K), idesc, k > 0 ? 1u : 0u);
}

/* 16 consecutive FP32 columns of this thread's lane, the load completed before returning (warp-collective:
 * the warp reconverges first) */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
	uint32_t r[16];
	__syncwarp();
	asm volatile(
			"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
			"tcgen05.wait::ld.sync.aligned;"
			: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
			"=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
			: "r"(taddr)
			: "memory");
#pragma unroll
	for(int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

/* tensor-memory address of (this warp's lane quadrant, column col) */
__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, int col) { return base + ((uint32_t) (32 * ((threadIdx.x >> 5) & 3)) << 16) + (uint32_t) col; }

/* ---------------------------------------------------------------- bf16 packing */
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
	const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
	return *(const uint32_t *) &h;
}

/* eight consecutive values of row r (columns k0..k0+7, k0 % 8 == 0) of a canonical matrix */
__device__ __forceinline__ void store_row8(__nv_bfloat16 *M, int r, int k0, int K, const float *v) {
	uint4 u;
	u.x = pack_bf16(v[0], v[1]);
	u.y = pack_bf16(v[2], v[3]);
	u.z = pack_bf16(v[4], v[5]);
	u.w = pack_bf16(v[6], v[7]);
	*(uint4 *) (M + cl_off(r, k0, K)) = u;
}

/* ---------------------------------------------------------------- MLP forward on a 128-row tile */
struct __align__(128) MlpFwdSmem {
	__nv_bfloat16 x[MLP_ROWS * MLP_K1];    /* layer-1 A (rows = particles) */
	__nv_bfloat16 h1[MLP_ROWS * MLP_HID];  /* layer-2 A */
	__nv_bfloat16 h2[MLP_ROWS * MLP_HID];  /* layer-3 A */
	unsigned char w[MLPI_FWD_BYTES];       /* W1, W2, W3 operand images */
	float b1[MLP_HID], b2[MLP_HID], b3[MLP_N3];
	uint64_t bar;
	uint32_t tmem;
	int err;
};

#define MLP_FWD_TMEM_COLS 128 /* D1 in columns 0..63, D2 in 64..127, D3 in 0..15 */

/* copy the operand image and biases (all threads) */
__device__ __forceinline__ void mlp_load_weights(MlpFwdSmem &S, const unsigned char *img) {
	const uint4 *src = (const uint4 *) img;
	uint4 *dst = (uint4 *) S.w;
	for(int i = threadIdx.x; i < MLPI_FWD_BYTES / 16; i += blockDim.x) dst[i] = src[i];
	const float *bias = (const float *) (img + MLPI_BIAS);
	for(int i = threadIdx.x; i < MLP_HID; i += blockDim.x) {
		S.b1[i] = bias[i];
		S.b2[i] = bias[MLP_HID + i];
	}
	if(threadIdx.x < MLP_N3) S.b3[threadIdx.x] = threadIdx.x < MLP_OUT ? bias[2 * MLP_HID + threadIdx.x] : 0.f;
}

/* setup: weights, barrier, tensor memory (all 128 threads; warp 0 allocates) */
__device__ __forceinline__ void mlp_fwd_begin(MlpFwdSmem &S, const unsigned char *img) {
	mlp_load_weights(S, img);
	if(threadIdx.x == 0) {
		mbar_init(&S.bar, 1);
		S.err = 0;
	}
	if(threadIdx.x < 32) tmem_alloc(&S.tmem, MLP_FWD_TMEM_COLS);
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
}

__device__ __forceinline__ void mlp_fwd_end(MlpFwdSmem &S) {
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if(threadIdx.x < 32) tmem_dealloc(S.tmem, MLP_FWD_TMEM_COLS);
}

/* write this thread's input row (36 FP32 features, row = threadIdx.x) */
__device__ __forceinline__ void mlp_put_x(MlpFwdSmem &S, const float *f) {
	const int r = threadIdx.x;
	float v[8];
#pragma unroll
	for(int c = 0; c < MLP_K1 / 8; c++) {
#pragma unroll
		for(int e = 0; e < 8; e++) v[e] = (8 * c + e < MLP_IN) ? f[8 * c + e] : 0.f;
		store_row8(S.x, r, 8 * c, MLP_K1, v);
	}
}

/* hidden-layer epilogue: row of D (64 columns at col0) + bias, ReLU, BF16 into the next A operand */
__device__ __forceinline__ void mlp_hidden_epilogue(uint32_t tbase, int col0, const float *bias, __nv_bfloat16 *out) {
	const int r = threadIdx.x;
#pragma unroll
	for(int c = 0; c < MLP_HID / 16; c++) {
		float v[16];
		tmem_ld16(tmem_lane_addr(tbase, col0 + 16 * c), v);
#pragma unroll
		for(int e = 0; e < 16; e++) v[e] = fmaxf(v[e] + bias[16 * c + e], 0.f);
		store_row8(out, r, 16 * c, MLP_HID, v);
		store_row8(out, r, 16 * c + 8, MLP_HID, v + 8);
	}
}

/* One forward pass of the tile (all 128 threads, after every row was written with mlp_put_x): the
 * thread's row of logits z[4] = W3 relu(W2 relu(W1 x + b1) + b2) + b3, BF16 operands, FP32 accumulation.
 * *phase is the barrier parity to wait for next (3 phases per call). Returns false on a barrier timeout. */
__device__ __forceinline__ bool mlp_forward_tile(MlpFwdSmem &S, uint32_t *phase, float *z) {
	const uint32_t t = S.tmem;
	bool ok = true;
	fence_async_smem();
	__syncthreads();
	if(S.err) { /* an earlier wait expired: no further tensor-core work in this CTA */
#pragma unroll
		for(int e = 0; e < MLP_OUT; e++) z[e] = 0.f;
		return false;
	}
	if(threadIdx.x == 0) {
		tc_fence_after();
		umma_gemm(t, S.x, S.w + MLPI_W1, MLP_K1, MLP_HID);
		umma_commit(&S.bar);
	}
	ok &= mbar_wait(&S.bar, *phase);
	*phase ^= 1u;
	tc_fence_after();
	mlp_hidden_epilogue(t, 0, S.b1, S.h1);
	fence_async_smem();
	tc_fence_before();
	__syncthreads();
	if(threadIdx.x == 0) {
		tc_fence_after();
		umma_gemm(t + 64, S.h1, S.w + MLPI_W2, MLP_HID, MLP_HID);
		umma_commit(&S.bar);
	}
	ok &= mbar_wait(&S.bar, *phase);
	*phase ^= 1u;
	tc_fence_after();
	mlp_hidden_epilogue(t, 64, S.b2, S.h2);
	fence_async_smem();
	tc_fence_before();
	__syncthreads();
	if(threadIdx.x == 0) {
		tc_fence_after();
		umma_gemm(t, S.h2, S.w + MLPI_W3, MLP_HID, MLP_N3);
		umma_commit(&S.bar);
	}
	ok &= mbar_wait(&S.bar, *phase);
	*phase ^= 1u;
	tc_fence_after();
	float v[16];
	tmem_ld16(tmem_lane_addr(t, 0), v);
#pragma unroll
	for(int e = 0; e < MLP_OUT; e++) z[e] = v[e] + S.b3[e];
	if(!ok) S.err = 1;
	tc_fence_before();
	__syncthreads();
	return ok;
}

/* ---------------------------------------------------------------- MLP forward, one warp and 32 rows */
/* The move kernel runs one warp per CTA (32 attempts, one per lane) so that a colour of a few thousand
 * attempts spreads over the whole GPU. The MMA is still M = 128: its A operand is a 128-row view whose
 * rows 32..127 run on into the following buffers (their D rows are never read), and the warp reads
 * tensor-memory lanes 0..31. D1, D2 and D3 reuse columns 0..63 (each is read before the next MMA). */
struct __align__(128) MlpWarpSmem {
	__nv_bfloat16 x[32 * MLP_K1];
	__nv_bfloat16 h1[32 * MLP_HID];
	__nv_bfloat16 h2[32 * MLP_HID];
	unsigned char w[MLPI_FWD_BYTES];
	float b1[MLP_HID], b2[MLP_HID], b3[MLP_N3];
	uint64_t bar;
	uint32_t tmem;
	int err;
};
#define MLP_WARP_TMEM_COLS 64
/* the 128-row A views of x, h1 and h2 stay inside the structure */
static_assert(offsetof(MlpWarpSmem, x) + 128 * MLP_K1 * 2 <= sizeof(MlpWarpSmem), "x view");
static_assert(offsetof(MlpWarpSmem, h1) + 128 * MLP_HID * 2 <= sizeof(MlpWarpSmem), "h1 view");
static_assert(offsetof(MlpWarpSmem, h2) + 128 * MLP_HID * 2 <= sizeof(MlpWarpSmem), "h2 view");

/* 16-byte asynchronous global -> shared copies (each thread waits for its own) */
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* setup (the whole warp) */
__device__ __forceinline__ void mlpw_begin(MlpWarpSmem &S, const unsigned char *img) {
	for(int i = threadIdx.x; i < MLPI_FWD_BYTES / 16; i += 32) cp_async16(S.w + 16 * i, img + 16 * i);
	const float *bias = (const float *) (img + MLPI_BIAS);
	for(int i = threadIdx.x; i < MLP_HID; i += 32) {
		S.b1[i] = bias[i];
		S.b2[i] = bias[MLP_HID + i];
	}
	if(threadIdx.x < MLP_N3) S.b3[threadIdx.x] = threadIdx.x < MLP_OUT ? bias[2 * MLP_HID + threadIdx.x] : 0.f;
	if(threadIdx.x == 0) {
		mbar_init(&S.bar, 1);
		S.err = 0;
	}
	tmem_alloc(&S.tmem, MLP_WARP_TMEM_COLS);
	cp_async_wait_all();
	tc_fence_before();
	__syncwarp();
	tc_fence_after();
}

__device__ __forceinline__ void mlpw_end(MlpWarpSmem &S) {
	tc_fence_before();
	__syncwarp();
	tc_fence_after();
	tmem_dealloc(S.tmem, MLP_WARP_TMEM_COLS);
}

__device__ __forceinline__ void mlpw_put_x(MlpWarpSmem &S, const float *f) {
	float v[8];
#pragma unroll
	for(int c = 0; c < MLP_K1 / 8; c++) {
#pragma unroll
		for(int e = 0; e < 8; e++) v[e] = (8 * c + e < MLP_IN) ? f[8 * c + e] : 0.f;
		store_row8(S.x, threadIdx.x, 8 * c, MLP_K1, v);
	}
}

/* lane 0 issues D[0..63] = A . B^T and commits; the warp waits. Once a wait has expired (S.err) the CTA
 * issues no further tensor-core work and its results are void (the host reports the error). */
__device__ __forceinline__ bool mlpw_mma(MlpWarpSmem &S, uint32_t *phase, const void *A, const void *B, int K, int N) {
	fence_async_smem();
	tc_fence_before();
	__syncwarp();
	tc_fence_after();
	if(S.err) return false;
	if(threadIdx.x == 0) {
		umma_gemm(S.tmem, A, B, K, N);
		umma_commit(&S.bar);
	}
	__syncwarp();
	bool ok = mbar_wait(&S.bar, *phase);
	ok = __all_sync(0xffffffffu, ok);
	*phase ^= 1u;
	if(!ok && threadIdx.x == 0) S.err = 1;
	__syncwarp();
	tc_fence_after();
	return ok;
}

/* logits of this lane's row (after every lane wrote its row with mlpw_put_x) */
__device__ __forceinline__ bool mlpw_forward(MlpWarpSmem &S, uint32_t *phase, float *z) {
	bool ok = mlpw_mma(S, phase, S.x, S.w + MLPI_W1, MLP_K1, MLP_HID);
	mlp_hidden_epilogue(S.tmem, 0, S.b1, S.h1);
	ok &= mlpw_mma(S, phase, S.h1, S.w + MLPI_W2, MLP_HID, MLP_HID);
	mlp_hidden_epilogue(S.tmem, 0, S.b2, S.h2);
	ok &= mlpw_mma(S, phase, S.h2, S.w + MLPI_W3, MLP_HID, MLP_N3);
	float v[16];
	tmem_ld16(tmem_lane_addr(S.tmem, 0), v);
#pragma unroll
	for(int e = 0; e < MLP_OUT; e++) z[e] = ok ? v[e] + S.b3[e] : 0.f;
	return ok;
}

/* ---------------------------------------------------------------- the proposal mixture */
#define MIX_K 4

/* mixture weights: pi = (1 - floor) softmax(z) + floor e_0 (component 0 = the plain move), FP32 with
 * explicitly rounded operations so every call site computes the same bits */
__device__ __forceinline__ void mix_weights(const float *z, float floor0, float *pi) {
	float m = z[0];
#pragma unroll
	for(int k = 1; k < MIX_K; k++) m = fmaxf(m, z[k]);
	float e[MIX_K], s = 0.f;
#pragma unroll
	for(int k = 0; k < MIX_K; k++) {
		e[k] = __expf(__fsub_rn(fmaxf(z[k], m - 30.f), m));
		s = __fadd_rn(s, e[k]);
	}
	const float inv = __fdiv_rn(__fsub_rn(1.f, floor0), s);
#pragma unroll
	for(int k = 0; k < MIX_K; k++) pi[k] = __fmul_rn(e[k], inv);
	pi[0] = __fadd_rn(pi[0], floor0);
}

#endif /* PPGPU_UMMA_CUH_ */
