/*
 * ppgpu_mlp.cu -- the learned proposal's network outside the move kernel: operand packing, a standalone
 * batched forward pass, and one training step (forward + backward + weight gradients) on the fifth-
 * generation tensor cores, BF16 operands and FP32 accumulation in tensor memory, plus the Adam update.
 *
 * Network (per particle): z = W3 relu(W2 relu(W1 x + b1) + b2) + b3, x = 36 FP32 features, z = the four
 * mixture logits. Training objective per sample (a contextual bandit over the four proposal components,
 * utilities u_k measured by the collection kernel):
 *     s = softmax(z),  pi = (1 - floor) s + floor e_0,  J = sum_k pi_k u_k + tau H(s),  H = -sum s log s
 * and the step minimises L = -(1/B) sum_samples J. dJ/dz_k = (1 - floor) s_k (u_k - sum_j s_j u_j)
 *                                                       - tau s_k (log s_k + H).
 * Backward, per 128-sample tile (all GEMMs tcgen05, M = 128):
 *     dH2 = dZ . W3           (A = dZ [128 x 16],  B = W3^T [64 x 16])
 *     dA2 = dH2 * [a2 > 0];  dH1 = dA2 . W2   (B = W2^T [64 x 64])
 *     dA1 = dH1 * [a1 > 0]
 *     [dW2 | . ; . | dW1] = [dA2^T ; dA1^T] . [H1^T ; X^T]^T     (one M = 128, N = 112, K = 128 GEMM)
 *     dW3 = dZ^T . H2                                            (rows 0..3 of an M = 128 GEMM, N = 80)
 * Bias gradients ride along as the GEMM column of a constant-one row of the B operand (X^T row 36,
 * H2^T row 64): column sums of the same BF16 values the weight gradients use. The weight-gradient
 * accumulators stay in tensor memory over all tiles a CTA takes in one step; one FP32 atomic per
 * parameter and CTA then adds them into the global gradient.
 */
#include "ppgpu_umma.cuh"

#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ppgpu.h"
#include "ppgpu_internal.h"

/* ------------------------------------------------------------------------------------------------ */
/* operand image                                                                                     */
/* ------------------------------------------------------------------------------------------------ */
__device__ __forceinline__ void put_bf16(unsigned char *img, int off_bytes, int r, int k, int K, float v) {
	((__nv_bfloat16 *) (img + off_bytes))[cl_off(r, k, K)] = __float2bfloat16_rn(v);
}

/* all threads of the CTA: FP32 parameters -> BF16 canonical operand images + FP32 biases */
__device__ void mlp_pack_block(const float *P, unsigned char *img) {
	for(int e = threadIdx.x; e < MLP_HID * MLP_K1; e += blockDim.x) {
		const int o = e / MLP_K1, i = e % MLP_K1;
		put_bf16(img, MLPI_W1, o, i, MLP_K1, i < MLP_IN ? P[MLP_OFF_W1 + o * MLP_IN + i] : 0.f);
	}
	for(int e = threadIdx.x; e < MLP_HID * MLP_HID; e += blockDim.x) {
		const int o = e / MLP_HID, i = e % MLP_HID;
		const float w = P[MLP_OFF_W2 + o * MLP_HID + i];
		put_bf16(img, MLPI_W2, o, i, MLP_HID, w);
		put_bf16(img, MLPI_W2T, i, o, MLP_HID, w);
	}
	for(int e = threadIdx.x; e < MLP_N3 * MLP_HID; e += blockDim.x) {
		const int o = e / MLP_HID, i = e % MLP_HID;
		const float w = o < MLP_OUT ? P[MLP_OFF_W3 + o * MLP_HID + i] : 0.f;
		put_bf16(img, MLPI_W3, o, i, MLP_HID, w);
		put_bf16(img, MLPI_W3T, i, o, MLP_N3, w);
	}
	float *bias = (float *) (img + MLPI_BIAS);
	for(int e = threadIdx.x; e < 2 * MLP_HID + 16; e += blockDim.x) {
		float v = 0.f;
		if(e < MLP_HID) v = P[MLP_OFF_B1 + e];
		else if(e < 2 * MLP_HID) v = P[MLP_OFF_B2 + e - MLP_HID];
		else if(e < 2 * MLP_HID + MLP_OUT) v = P[MLP_OFF_B3 + e - 2 * MLP_HID];
		bias[e] = v;
	}
}

__global__ void k_mlp_pack(const float *P, unsigned char *img) { mlp_pack_block(P, img); }

/* ------------------------------------------------------------------------------------------------ */
/* standalone forward: z[n][4] of x[n][36]                                                           */
/* ------------------------------------------------------------------------------------------------ */
__global__ void __launch_bounds__(MLP_ROWS) k_mlp_forward(const unsigned char *img, const float *x, int n, float *z, int *err) {
	extern __shared__ __align__(128) unsigned char smem_raw[];
	MlpFwdSmem &S = *(MlpFwdSmem *) smem_raw;
	mlp_fwd_begin(S, img);
	uint32_t phase = 0;
	const int ntiles = (n + MLP_ROWS - 1) / MLP_ROWS;
	for(int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		const int s = tile * MLP_ROWS + threadIdx.x;
		float f[MLP_IN];
#pragma unroll
		for(int i = 0; i < MLP_IN; i++) f[i] = s < n ? x[(size_t) s * MLP_IN + i] : 0.f;
		mlp_put_x(S, f);
		float zz[MLP_OUT];
		mlp_forward_tile(S, &phase, zz);
		if(s < n)
#pragma unroll
			for(int k = 0; k < MLP_OUT; k++) z[(size_t) s * MLP_OUT + k] = zz[k];
	}
	mlp_fwd_end(S);
	if(threadIdx.x == 0 && S.err) atomicExch(err, 1);
}

/* ------------------------------------------------------------------------------------------------ */
/* training step                                                                                     */
/* ------------------------------------------------------------------------------------------------ */
#define MLP_WG_N 112  /* weight-gradient GEMM: N = 64 (H1^T) + 48 (X^T) */
#define MLP_W3G_N 80  /* dW3 GEMM: N = 64 (H2^T) + ones row + padding */
#define MLP_ONES_X 100 /* row of the weight-gradient B operand holding ones (X^T row 36) */

struct __align__(128) MlpTrainSmem {
	__nv_bfloat16 x[MLP_ROWS * MLP_K1];
	__nv_bfloat16 h1[MLP_ROWS * MLP_HID];
	__nv_bfloat16 h2[MLP_ROWS * MLP_HID];
	__nv_bfloat16 dz[MLP_ROWS * MLP_N3];
	__nv_bfloat16 da2[MLP_ROWS * MLP_HID];
	__nv_bfloat16 aw[128 * MLP_ROWS];        /* rows 0-63 dA2^T, rows 64-127 dA1^T (K = samples) */
	__nv_bfloat16 dzt[MLP_N3 * MLP_ROWS];    /* dZ^T: rows 0-15 of the dW3 GEMM's 128-row A view ... */
	__nv_bfloat16 bw[MLP_WG_N * MLP_ROWS];   /* ... which continues over this buffer (rows 16-127 unused) */
	__nv_bfloat16 b3m[MLP_W3G_N * MLP_ROWS]; /* rows 0-63 H2^T, row 64 ones, rows 65-79 zero */
	unsigned char w[MLPI_BIAS];
	float b1[MLP_HID], b2[MLP_HID], b3[MLP_N3];
	double obj[4];
	uint64_t bar;
	uint32_t tmem;
	int err;
};
static_assert(offsetof(MlpTrainSmem, bw) == offsetof(MlpTrainSmem, dzt) + sizeof(((MlpTrainSmem *) 0)->dzt), "dZ^T view must run into bw");
static_assert(sizeof(((MlpTrainSmem *) 0)->dzt) + sizeof(((MlpTrainSmem *) 0)->bw) == 128 * MLP_ROWS * 2, "dW3 A view spans exactly 128 rows");

/* tensor-memory columns of the training kernel (512 allocated: one CTA per SM by shared memory) */
#define TT_D1 0     /* layer 1, then dH2 */
#define TT_D2 64    /* layer 2, then dH1 */
#define TT_D3 128   /* layer 3 */
#define TT_G3 160   /* dW3 | db3 accumulator, 80 columns */
#define TT_GW 256   /* dW2 | dW1 | db accumulator, 112 columns */
#define TT_COLS 512

__device__ __forceinline__ void put_t(__nv_bfloat16 *M, int row, int col, float v) { M[cl_off(row, col, MLP_ROWS)] = __float2bfloat16_rn(v); }

/* one commit + wait; false on timeout (the CTA then stops issuing tensor-core work: S.err) */
__device__ __forceinline__ bool tc_sync(MlpTrainSmem &S, uint32_t &phase) {
	if(threadIdx.x == 0) umma_commit(&S.bar);
	bool ok = mbar_wait(&S.bar, phase);
	phase ^= 1u;
	if(!ok) S.err = 1;
	__syncthreads();
	ok = S.err == 0;
	tc_fence_after();
	return ok;
}

/* make this thread's shared-memory operand writes visible and hand over to the issuing thread */
__device__ __forceinline__ void operands_ready() {
	fence_async_smem();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
}

/* objective gradient of one sample (FP32), returns J */
__device__ __forceinline__ float sample_grad(const float *z, const float *u, float floor0, float tau, float inv_batch, float *dz) {
	float m = z[0];
#pragma unroll
	for(int k = 1; k < MLP_OUT; k++) m = fmaxf(m, z[k]);
	float e[MLP_OUT], S = 0.f;
#pragma unroll
	for(int k = 0; k < MLP_OUT; k++) {
		e[k] = expf(z[k] - m);
		S += e[k];
	}
	const float lS = logf(S);
	float s[MLP_OUT], ls[MLP_OUT], H = 0.f, ub = 0.f, J = 0.f;
#pragma unroll
	for(int k = 0; k < MLP_OUT; k++) {
		s[k] = e[k] / S;
		ls[k] = (z[k] - m) - lS;
		H -= s[k] * ls[k];
		ub += s[k] * u[k];
		J += ((1.f - floor0) * s[k] + (k == 0 ? floor0 : 0.f)) * u[k];
	}
	J += tau * H;
#pragma unroll
	for(int k = 0; k < MLP_OUT; k++) {
		const float g = (1.f - floor0) * s[k] * (u[k] - ub) - tau * s[k] * (ls[k] + H);
		dz[k] = -g * inv_batch;
	}
	return J;
}

/* Gradient of the batch formed by tiles tile_ids[c * tiles_per_cta + j] (CTA c), added into grad[] (FP32
 * atomics, layout of the master parameters); objective sum into *objective. */
__global__ void __launch_bounds__(MLP_ROWS, 1) k_mlp_train(const unsigned char *img, const float *samples, int n_samples, const int *tile_ids, int n_tiles,
		int tiles_per_cta, float floor0, float tau, float inv_batch, float *grad, double *objective, int *err) {
	extern __shared__ __align__(128) unsigned char smem_raw[];
	MlpTrainSmem &S = *(MlpTrainSmem *) smem_raw;
	const int t = threadIdx.x;
	{
		const uint4 *src = (const uint4 *) img;
		uint4 *dst = (uint4 *) S.w;
		for(int i = t; i < MLPI_BIAS / 16; i += blockDim.x) dst[i] = src[i];
		const float *bias = (const float *) (img + MLPI_BIAS);
		if(t < MLP_HID) {
			S.b1[t] = bias[t];
			S.b2[t] = bias[MLP_HID + t];
		}
		if(t < MLP_N3) S.b3[t] = t < MLP_OUT ? bias[2 * MLP_HID + t] : 0.f;
		if(t < 4) S.obj[t] = 0.;
	}
	if(t == 0) {
		mbar_init(&S.bar, 1);
		S.err = 0;
	}
	if(t < 32) tmem_alloc(&S.tmem, TT_COLS);
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tm = S.tmem;
	uint32_t phase = 0;
	bool ok = true;
	int ntile_done = 0;
	float J_acc = 0.f;
	for(int j = 0; j < tiles_per_cta; j++) {
		const int ti = blockIdx.x * tiles_per_cta + j;
		if(ti >= n_tiles) break;
		const int s = tile_ids[ti] * MLP_ROWS + t;
		const bool valid = s < n_samples;
		float f[MLP_IN], u[MLP_OUT];
#pragma unroll
		for(int i = 0; i < MLP_IN; i++) f[i] = valid ? samples[(size_t) s * MLP_SAMPLE + i] : 0.f;
#pragma unroll
		for(int k = 0; k < MLP_OUT; k++) u[k] = valid ? samples[(size_t) s * MLP_SAMPLE + MLP_IN + k] : 0.f;
		/* X row (layer-1 A) and X^T column (weight-gradient B rows 64..111, row 100 = ones) */
		{
			float v[8];
#pragma unroll
			for(int c = 0; c < MLP_K1 / 8; c++) {
#pragma unroll
				for(int e = 0; e < 8; e++) v[e] = (8 * c + e < MLP_IN) ? f[8 * c + e] : 0.f;
				store_row8(S.x, t, 8 * c, MLP_K1, v);
			}
#pragma unroll
			for(int i = 0; i < MLP_K1; i++) put_t(S.bw, MLP_HID + i, t, i < MLP_IN ? f[i] : (i == MLP_IN ? 1.f : 0.f));
		}
		operands_ready();
		if(t == 0 && !S.err) umma_gemm(tm + TT_D1, S.x, S.w + MLPI_W1, MLP_K1, MLP_HID);
		ok &= tc_sync(S, phase);
		/* layer-1 epilogue: H1 row, H1^T column, ReLU mask */
		uint64_t mask1 = 0ull, mask2 = 0ull;
#pragma unroll
		for(int c = 0; c < MLP_HID / 16; c++) {
			float v[16];
			tmem_ld16(tmem_lane_addr(tm, TT_D1 + 16 * c), v);
#pragma unroll
			for(int e = 0; e < 16; e++) {
				const float a = v[e] + S.b1[16 * c + e];
				mask1 |= (uint64_t) (a > 0.f) << (16 * c + e);
				v[e] = fmaxf(a, 0.f);
				put_t(S.bw, 16 * c + e, t, v[e]);
			}
			store_row8(S.h1, t, 16 * c, MLP_HID, v);
			store_row8(S.h1, t, 16 * c + 8, MLP_HID, v + 8);
		}
		operands_ready();
		if(t == 0 && !S.err) umma_gemm(tm + TT_D2, S.h1, S.w + MLPI_W2, MLP_HID, MLP_HID);
		ok &= tc_sync(S, phase);
#pragma unroll
		for(int c = 0; c < MLP_HID / 16; c++) {
			float v[16];
			tmem_ld16(tmem_lane_addr(tm, TT_D2 + 16 * c), v);
#pragma unroll
			for(int e = 0; e < 16; e++) {
				const float a = v[e] + S.b2[16 * c + e];
				mask2 |= (uint64_t) (a > 0.f) << (16 * c + e);
				v[e] = fmaxf(a, 0.f);
				put_t(S.b3m, 16 * c + e, t, v[e]);
			}
			store_row8(S.h2, t, 16 * c, MLP_HID, v);
			store_row8(S.h2, t, 16 * c + 8, MLP_HID, v + 8);
		}
#pragma unroll
		for(int i = MLP_HID; i < MLP_W3G_N; i++) put_t(S.b3m, i, t, i == MLP_HID ? 1.f : 0.f);
		operands_ready();
		if(t == 0 && !S.err) umma_gemm(tm + TT_D3, S.h2, S.w + MLPI_W3, MLP_HID, MLP_N3);
		ok &= tc_sync(S, phase);
		float z[MLP_OUT], dz[MLP_OUT];
		{
			float v[16];
			tmem_ld16(tmem_lane_addr(tm, TT_D3), v);
#pragma unroll
			for(int k = 0; k < MLP_OUT; k++) z[k] = v[k] + S.b3[k];
		}
		const float J = sample_grad(z, u, floor0, tau, inv_batch, dz);
		if(valid) J_acc += J;
		else
#pragma unroll
			for(int k = 0; k < MLP_OUT; k++) dz[k] = 0.f;
		{
			float v[16];
#pragma unroll
			for(int e = 0; e < 16; e++) v[e] = e < MLP_OUT ? dz[e] : 0.f;
			store_row8(S.dz, t, 0, MLP_N3, v);
			store_row8(S.dz, t, 8, MLP_N3, v + 8);
#pragma unroll
			for(int e = 0; e < MLP_N3; e++) put_t(S.dzt, e, t, v[e]);
		}
		operands_ready();
		if(t == 0 && !S.err) umma_gemm(tm + TT_D1, S.dz, S.w + MLPI_W3T, MLP_N3, MLP_HID);
		ok &= tc_sync(S, phase);
		/* dA2 = dH2 * relu'(a2): row (A of dH1) and column (weight-gradient A rows 0..63) */
#pragma unroll
		for(int c = 0; c < MLP_HID / 16; c++) {
			float v[16];
			tmem_ld16(tmem_lane_addr(tm, TT_D1 + 16 * c), v);
#pragma unroll
			for(int e = 0; e < 16; e++) {
				v[e] = ((mask2 >> (16 * c + e)) & 1ull) ? v[e] : 0.f;
				put_t(S.aw, 16 * c + e, t, v[e]);
			}
			store_row8(S.da2, t, 16 * c, MLP_HID, v);
			store_row8(S.da2, t, 16 * c + 8, MLP_HID, v + 8);
		}
		operands_ready();
		if(t == 0 && !S.err) umma_gemm(tm + TT_D2, S.da2, S.w + MLPI_W2T, MLP_HID, MLP_HID);
		ok &= tc_sync(S, phase);
#pragma unroll
		for(int c = 0; c < MLP_HID / 16; c++) {
			float v[16];
			tmem_ld16(tmem_lane_addr(tm, TT_D2 + 16 * c), v);
#pragma unroll
			for(int e = 0; e < 16; e++) put_t(S.aw, MLP_HID + 16 * c + e, t, ((mask1 >> (16 * c + e)) & 1ull) ? v[e] : 0.f);
		}
		operands_ready();
		if(t == 0 && !S.err) {
			const uint32_t a = smem_u32(S.aw), b = smem_u32(S.bw), a3 = smem_u32(S.dzt), b3 = smem_u32(S.b3m);
			const uint32_t idw = umma_idesc_bf16(128, MLP_WG_N), id3 = umma_idesc_bf16(128, MLP_W3G_N);
			for(int k = 0; k < MLP_ROWS / 16; k++) {
				const uint32_t acc = (ntile_done > 0 || k > 0) ? 1u : 0u;
				umma_bf16(tm + TT_GW, umma_kmajor(a + 256u * k, MLP_ROWS), umma_kmajor(b + 256u * k, MLP_ROWS), idw, acc);
				umma_bf16(tm + TT_G3, umma_kmajor(a3 + 256u * k, MLP_ROWS), umma_kmajor(b3 + 256u * k, MLP_ROWS), id3, acc);
			}
		}
		ok &= tc_sync(S, phase); /* the operands of the next tile overwrite these buffers */
		ntile_done++;
	}
	/* weight gradients: row m of the accumulators */
	if(ntile_done > 0) {
		float v[16];
		if(t < MLP_HID) { /* dW2 row t, db2[t] */
#pragma unroll 1
			for(int c = 0; c < MLP_HID / 16; c++) {
				tmem_ld16(tmem_lane_addr(tm, TT_GW + 16 * c), v);
#pragma unroll
				for(int e = 0; e < 16; e++) atomicAdd(grad + MLP_OFF_W2 + t * MLP_HID + 16 * c + e, v[e]);
			}
		}
		else { /* dW1 row t - 64 */
			const int o = t - MLP_HID;
#pragma unroll 1
			for(int c = 0; c < MLP_K1 / 16; c++) {
				tmem_ld16(tmem_lane_addr(tm, TT_GW + MLP_HID + 16 * c), v);
#pragma unroll
				for(int e = 0; e < 16; e++)
					if(16 * c + e < MLP_IN) atomicAdd(grad + MLP_OFF_W1 + o * MLP_IN + 16 * c + e, v[e]);
			}
		}
		/* bias column (every thread loads: tcgen05.ld is warp-collective) */
		tmem_ld16(tmem_lane_addr(tm, TT_GW + MLP_HID + 32), v); /* columns 96..111, ones at 100 */
		atomicAdd(grad + (t < MLP_HID ? MLP_OFF_B2 + t : MLP_OFF_B1 + (t - MLP_HID)), v[MLP_ONES_X - MLP_HID - 32]);
#pragma unroll 1
		for(int c = 0; c < MLP_W3G_N / 16; c++) {
			tmem_ld16(tmem_lane_addr(tm, TT_G3 + 16 * c), v);
			if(t < MLP_OUT)
#pragma unroll
				for(int e = 0; e < 16; e++) {
					const int col = 16 * c + e;
					if(col < MLP_HID) atomicAdd(grad + MLP_OFF_W3 + t * MLP_HID + col, v[e]);
					else if(col == MLP_HID) atomicAdd(grad + MLP_OFF_B3 + t, v[e]);
				}
		}
	}
	/* objective */
	{
		float Jw = J_acc;
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) Jw += __shfl_xor_sync(0xffffffffu, Jw, o);
		if((t & 31) == 0) S.obj[t >> 5] = (double) Jw;
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if(t == 0) {
		if(ntile_done > 0) atomicAdd(objective, S.obj[0] + S.obj[1] + S.obj[2] + S.obj[3]);
		if(!ok) atomicExch(err, 1);
	}
	if(t < 32) tmem_dealloc(tm, TT_COLS);
}

/* Adam on the FP32 master parameters (one CTA), gradient buffer zeroed, operand image rebuilt */
__global__ void k_mlp_adam(float *P, float *grad, float *m1, float *m2, unsigned char *img, int step, float lr, float beta1, float beta2, float eps) {
	const float c1 = 1.f - powf(beta1, (float) step), c2 = 1.f - powf(beta2, (float) step);
	for(int i = threadIdx.x; i < MLP_NPARAMS; i += blockDim.x) {
		const float g = grad[i];
		grad[i] = 0.f;
		const float a = beta1 * m1[i] + (1.f - beta1) * g, b = beta2 * m2[i] + (1.f - beta2) * g * g;
		m1[i] = a;
		m2[i] = b;
		P[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
	}
	__syncthreads();
	mlp_pack_block(P, img);
}

/* ------------------------------------------------------------------------------------------------ */
/* launchers (used by the engine, ppgpu_host.c) and standalone entry points                         */
/* ------------------------------------------------------------------------------------------------ */
extern "C" int ppi_mlp_pack(const float *P_dev, unsigned char *img_dev, cudaStream_t s) {
	k_mlp_pack<<<1, 256, 0, s>>>(P_dev, img_dev);
	return (int) cudaGetLastError();
}

static int mlp_attr_done = 0;
static int mlp_set_attrs(void) {
	if(mlp_attr_done) return 0;
	cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(MlpFwdSmem));
	if(e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(MlpTrainSmem));
	if(e == cudaSuccess) mlp_attr_done = 1;
	return (int) e;
}

extern "C" int ppi_mlp_forward(const unsigned char *img, const float *x_dev, int n, float *z_dev, int *err_dev, cudaStream_t s) {
	int e = mlp_set_attrs();
	if(e) return e;
	const int ntiles = (n + MLP_ROWS - 1) / MLP_ROWS;
	if(ntiles == 0) return 0;
	k_mlp_forward<<<ntiles, MLP_ROWS, sizeof(MlpFwdSmem), s>>>(img, x_dev, n, z_dev, err_dev);
	return (int) cudaGetLastError();
}

extern "C" int ppi_mlp_train_step(const unsigned char *img, const float *samples, int n_samples, const int *tile_ids, int n_tiles, int tiles_per_cta, float floor0,
		float tau, float inv_batch, float *grad, double *objective, int *err_dev, cudaStream_t s) {
	int e = mlp_set_attrs();
	if(e) return e;
	const int grid = (n_tiles + tiles_per_cta - 1) / tiles_per_cta;
	if(grid == 0) return 0;
	k_mlp_train<<<grid, MLP_ROWS, sizeof(MlpTrainSmem), s>>>(img, samples, n_samples, tile_ids, n_tiles, tiles_per_cta, floor0, tau, inv_batch, grad, objective, err_dev);
	return (int) cudaGetLastError();
}

extern "C" int ppi_mlp_adam(float *P, float *grad, float *m1, float *m2, unsigned char *img, int step, float lr, cudaStream_t s) {
	k_mlp_adam<<<1, 256, 0, s>>>(P, grad, m1, m2, img, step, lr, 0.9f, 0.999f, 1e-8f);
	return (int) cudaGetLastError();
}

/* ---- standalone C-ABI: the network on caller-provided host arrays (allocates device memory) ---- */
struct MlpScratch {
	float *P;
	unsigned char *img;
	float *a, *b, *g;
	int *ids, *err;
	double *obj;
};

static void mlp_free(MlpScratch &m) {
	cudaFree(m.P);
	cudaFree(m.img);
	cudaFree(m.a);
	cudaFree(m.b);
	cudaFree(m.g);
	cudaFree(m.ids);
	cudaFree(m.err);
	cudaFree(m.obj);
}

#define MLP_TRY(x)                         \
	do {                                   \
		cudaError_t e_ = (x);              \
		if(e_ != cudaSuccess) {            \
			mlp_free(m);                   \
			return PP_ERR_CUDA;            \
		}                                  \
	} while(0)

extern "C" int pp_mlp_forward(const float *params, int n, const float *x, float *z) {
	if(!params || n < 0 || (n > 0 && (!x || !z))) return PP_ERR_ARG;
	if(n == 0) return PP_OK;
	MlpScratch m;
	memset(&m, 0, sizeof(m));
	MLP_TRY(cudaMalloc(&m.P, MLP_NPARAMS * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.img, MLPI_BYTES));
	MLP_TRY(cudaMalloc(&m.a, (size_t) n * MLP_IN * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.b, (size_t) n * MLP_OUT * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.err, sizeof(int)));
	MLP_TRY(cudaMemset(m.err, 0, sizeof(int)));
	MLP_TRY(cudaMemcpy(m.P, params, MLP_NPARAMS * sizeof(float), cudaMemcpyHostToDevice));
	MLP_TRY(cudaMemcpy(m.a, x, (size_t) n * MLP_IN * sizeof(float), cudaMemcpyHostToDevice));
	MLP_TRY((cudaError_t) ppi_mlp_pack(m.P, m.img, 0));
	MLP_TRY((cudaError_t) ppi_mlp_forward(m.img, m.a, n, m.b, m.err, 0));
	MLP_TRY(cudaMemcpy(z, m.b, (size_t) n * MLP_OUT * sizeof(float), cudaMemcpyDeviceToHost));
	int err = 0;
	MLP_TRY(cudaMemcpy(&err, m.err, sizeof(int), cudaMemcpyDeviceToHost));
	mlp_free(m);
	return err ? PP_ERR_CUDA : PP_OK;
}

extern "C" int pp_mlp_grad(const float *params, int n, const float *samples, double floor0, double tau, int tiles_per_cta, float *grad, double *objective) {
	if(!params || n <= 0 || !samples || !grad || tiles_per_cta <= 0) return PP_ERR_ARG;
	MlpScratch m;
	memset(&m, 0, sizeof(m));
	const int ntiles = (n + MLP_ROWS - 1) / MLP_ROWS;
	int *ids = (int *) malloc(ntiles * sizeof(int));
	if(!ids) return PP_ERR_ARG;
	for(int i = 0; i < ntiles; i++) ids[i] = i;
	MLP_TRY(cudaMalloc(&m.P, MLP_NPARAMS * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.img, MLPI_BYTES));
	MLP_TRY(cudaMalloc(&m.a, (size_t) n * MLP_SAMPLE * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.g, MLP_NPARAMS * sizeof(float)));
	MLP_TRY(cudaMalloc(&m.ids, ntiles * sizeof(int)));
	MLP_TRY(cudaMalloc(&m.err, sizeof(int)));
	MLP_TRY(cudaMalloc(&m.obj, sizeof(double)));
	MLP_TRY(cudaMemset(m.err, 0, sizeof(int)));
	MLP_TRY(cudaMemset(m.obj, 0, sizeof(double)));
	MLP_TRY(cudaMemset(m.g, 0, MLP_NPARAMS * sizeof(float)));
	MLP_TRY(cudaMemcpy(m.P, params, MLP_NPARAMS * sizeof(float), cudaMemcpyHostToDevice));
	MLP_TRY(cudaMemcpy(m.a, samples, (size_t) n * MLP_SAMPLE * sizeof(float), cudaMemcpyHostToDevice));
	MLP_TRY(cudaMemcpy(m.ids, ids, ntiles * sizeof(int), cudaMemcpyHostToDevice));
	free(ids);
	MLP_TRY((cudaError_t) ppi_mlp_pack(m.P, m.img, 0));
	MLP_TRY((cudaError_t) ppi_mlp_train_step(m.img, m.a, n, m.ids, ntiles, tiles_per_cta, (float) floor0, (float) tau, 1.f / (float) n, m.g, m.obj, m.err, 0));
	MLP_TRY(cudaMemcpy(grad, m.g, MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost));
	double obj = 0.;
	int err = 0;
	MLP_TRY(cudaMemcpy(&obj, m.obj, sizeof(double), cudaMemcpyDeviceToHost));
	MLP_TRY(cudaMemcpy(&err, m.err, sizeof(int), cudaMemcpyDeviceToHost));
	if(objective) *objective = obj / n;
	mlp_free(m);
	return err ? PP_ERR_CUDA : PP_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* failure detection of the tensor-core waits                                                        */
/* ------------------------------------------------------------------------------------------------ */
/* One warp waits, the way tc_sync waits for a commit, on an mbarrier of expected count 1. With arrive = 1
 * thread 0 arrives first and the wait completes; with arrive = 0 nothing arrives and no tensor-core work is
 * issued, so the wait runs out after limit cycles. out[0] = 1 when any lane gave up, out[1] = the longest
 * wait in cycles. */
__global__ void k_mbar_wait_test(long long limit, int arrive, long long *out) {
	__shared__ uint64_t bar;
	__shared__ int gave_up;
	__shared__ unsigned long long longest;
	if(threadIdx.x == 0) {
		mbar_init(&bar, 1);
		gave_up = 0;
		longest = 0ull;
	}
	__syncthreads();
	if(arrive && threadIdx.x == 0) mbar_arrive(&bar);
	const long long t0 = clock64();
	const bool ok = mbar_wait(&bar, 0u, limit);
	const long long dt = clock64() - t0;
	if(!ok) gave_up = 1;
	atomicMax(&longest, (unsigned long long) dt);
	__syncthreads();
	if(threadIdx.x == 0) {
		out[0] = gave_up;
		out[1] = (long long) longest;
	}
}

extern "C" int pp_mlp_wait_test(long long limit_cycles, int arrive, int *timed_out, long long *cycles) {
	if(limit_cycles <= 0 || limit_cycles > UMMA_WAIT_CYCLES || (arrive != 0 && arrive != 1)) return PP_ERR_ARG;
	long long *out = NULL, h[2] = {0, 0};
	if(cudaMalloc(&out, sizeof(h)) != cudaSuccess) return PP_ERR_CUDA;
	k_mbar_wait_test<<<1, 32>>>(limit_cycles, arrive, out);
	cudaError_t e = cudaGetLastError();
	if(e == cudaSuccess) e = cudaMemcpy(h, out, sizeof(h), cudaMemcpyDeviceToHost);
	cudaFree(out);
	if(e != cudaSuccess) return PP_ERR_CUDA;
	if(timed_out) *timed_out = (int) h[0];
	if(cycles) *cycles = h[1];
	return h[0] ? PP_ERR_CUDA : PP_OK;
}
