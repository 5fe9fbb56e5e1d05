/*
 * ppgpu_kernels.cu -- sm_103a kernels of the roto-translation Monte Carlo engine (global checkerboard).
 *
 * Every `resort_every` rounds each replica gets a new cell grid (even number of cells per axis, edge >=
 * r_cut, random origin shift) and the particles are counting-sorted into cell order as FP32 working
 * records (spos 16 B + sori 48 B) rebuilt from the FP64 canonical state:
 *   k_grid, k_assign, k_scan, k_scatter, k_cellfin (deterministic in-cell order, colour lists)
 * and every particle's neighbour list for the epoch is built (k_nlist: the candidates that can come within
 * r_cut before the next re-sort).
 * One round = the 8 colours of the 2x2x2 checkerboard, one launch each (k_colour): every non-empty
 * cell of the colour gets one roto-translation attempt on a uniformly chosen particle of the cell
 * (MC_move_rototranslate, MC.c:311-340). A warp takes 64 attempts and flattens their neighbour pairs
 * (from the lists, or from the 27 cells) into one shared pair list that its lanes walk 32 pairs per step.
 * Same-colour cells are never adjacent and a move that leaves its cell is rejected, so concurrent moves
 * never interact and the cell lists stay valid for the whole epoch. The pair test is FP32 with an FP64
 * re-evaluation inside the guard band, bit-identical to MC_would_interact (MC.c:232-266). Accepted moves
 * update the FP64 state with FP64 arithmetic (r + disp, q (x) dq) and the FP32 record in place.
 * k_energy: energy from scratch (per-particle bonds/overlaps, output.c:213-268); the candidate box of the
 * sweep's NPT volume move (MC.c:487-495) or NVT box-shape move (MC.c:554-560) from the epoch's flat pair
 * list (k_energy_vol_pairs, k_vol_unsure) or, without lists, per particle (k_energy_vol); k_vol_*: the
 * volume and box-shape moves (MC.c:450-513, 515-585). The sort, the volume move and the colours of a round
 * are chained by programmatic dependent launch (grid_dep_wait).
 */
#include "ppgpu.h"
#include "ppgpu_internal.h"
#include "ppgpu_umma.cuh"

#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11)   */
/* ------------------------------------------------------------------------------------------------ */
struct U4 {
	uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
	for(int i = 0; i < 10; i++) {
		uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
		uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
		c = U4{ hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0 };
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	return c;
}

/* counter layout: x = sweep (low 32 bits), y = sweep (high bits) << 8 | tag, z = cell / item, w = sub-index.
 * The key is the replica's own seed, so a replica's stream does not depend on its position in a batch. */
#define TAG_PLAN 1u
#define TAG_CELLN 2u
#define TAG_MOVE 3u

__device__ __forceinline__ U4 rng(const ppi_rparams &rp, long long sweep, int replica, uint32_t tag, uint32_t item, uint32_t sub) {
	(void) replica;
	return philox(U4{ (uint32_t) sweep, ((uint32_t) ((unsigned long long) sweep >> 32) << 8) | tag, item, sub }, (uint32_t) rp.seed, (uint32_t) (rp.seed >> 32));
}

/* index of a launch: a non-negative argument is the index itself, a negative one (-1 - k) the k-th after
 * the device counter base (the launches of a captured sweep graph) */
__device__ __forceinline__ long long ctr_index(long long arg, long long base) { return arg >= 0 ? arg : base + (-1 - arg); }

/* colour of slot ci in round `round`: the host's colour_order (ppgpu_host.c), a Fisher-Yates shuffle driven
 * by splitmix64 of the round index, evaluated on the device for graph launches */
__device__ __forceinline__ int colour_at(long long round, int ci) {
	uint64_t z = (uint64_t) round * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
	int col[8];
#pragma unroll
	for(int i = 0; i < 8; i++) col[i] = i;
#pragma unroll
	for(int i = 7; i > 0; i--) {
		z += 0x9E3779B97F4A7C15ULL;
		uint64_t x = z;
		x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
		x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
		x ^= x >> 31;
		const int j = (int) (x % (uint64_t) (i + 1));
		const int t = col[i];
		col[i] = col[j];
		col[j] = t;
	}
	return col[ci & 7];
}

__device__ __forceinline__ float u01(uint32_t v) { return (float) (v >> 8) * 0x1p-24f; } /* [0, 1) */
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) { return (double) (((uint64_t) a << 21) | (b >> 11)) * 0x1p-53; }

/* Programmatic dependent launch. A kernel launched with programmatic stream serialisation may start
 * before its predecessor completes: grid_dep_wait blocks until the predecessor has completed and its
 * writes are visible, grid_dep_release lets the next such launch begin. Both are no-ops in an ordinary
 * launch. The colour passes draw their first proposals (which read only their own movers, untouched by
 * the previous colour, and the epoch's colour and neighbour lists) before the wait; the chained kernels
 * of the sort and of the volume move wait first. */
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

/* L2 eviction priorities for the colour pass: the FP32 working records (spos, sori), which every colour
 * launch gathers again, are loaded with evict_last; the per-launch streams (colour lists, neighbour
 * lists) with evict_first, so that they do not push the records out of L2 between launches */
#ifndef PPI_L2HINT
#define PPI_L2HINT 1
#endif
__device__ __forceinline__ uint64_t l2_keep() {
	uint64_t p;
	asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ uint64_t l2_stream() {
	uint64_t p;
	asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ float4 ld_keep(const float4 *a) {
#if PPI_L2HINT
	float4 v;
	asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(a), "l"(l2_keep()));
	return v;
#else
	return *a;
#endif
}

__device__ __forceinline__ int4 ld_stream(const int4 *a) {
#if PPI_L2HINT
	int4 v;
	asm volatile("ld.global.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(a), "l"(l2_stream()));
	return v;
#else
	return *a;
#endif
}

/* ------------------------------------------------------------------------------------------------ */
/* Reference-exact FP64 pair test: MC_would_interact (MC.c:232-266) with the patches of              */
/* MATRIX_VECTOR_MULTIPLICATION (utils.h:17-21). Every operation is an explicitly rounded IEEE        */
/* operation, so nothing is contracted into an FMA and the result equals the reference's bit for bit. */
/* ------------------------------------------------------------------------------------------------ */
/* patch i of an orientation: R . base_i with the MATRIX_VECTOR_MULTIPLICATION order (utils.h:17-21) */
__device__ __forceinline__ void patch64(const double *R, const double *b, double *P) {
#pragma unroll
	for(int k = 0; k < 3; k++) P[k] = __dadd_rn(__dadd_rn(__dmul_rn(R[3 * k + 0], b[0]), __dmul_rn(R[3 * k + 1], b[1])), __dmul_rn(R[3 * k + 2], b[2]));
}

__device__ __forceinline__ double scalar64(const double *a, const double *b) {
	return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

/* MC_would_interact (MC.c:232-266) for p = (rp, Rp) and q = (rq, Rq): returns -1 overlap, 0 no bond,
 * 1 bond; optional diagnostics (dist2, max p cosine, max q cosine). Patches are formed one at a time
 * from the orientations (same operations as the stored patches of the reference), which keeps this cold
 * path light on registers. */
__device__ __noinline__ int interact64(const double *rp, const double *Rp, const double *rq, const double *Rq, const double (*base)[3], const double *box, double sqr_rcut,
		double cosmax, double *o_dist2, double *o_pmax, double *o_qmax) {
	double d[3];
#pragma unroll 1
	for(int k = 0; k < 3; k++) {
		d[k] = __dsub_rn(rq[k], rp[k]);
		d[k] = __dsub_rn(d[k], __dmul_rn(box[k], rint(__ddiv_rn(d[k], box[k]))));
	}
	double dist2 = scalar64(d, d);
	if(o_dist2) *o_dist2 = dist2;
	if(dist2 < 1.) return -1;
	int res = 0;
	if(dist2 < sqr_rcut) {
		double norm = __dsqrt_rn(dist2);
		d[0] = __ddiv_rn(d[0], norm);
		d[1] = __ddiv_rn(d[1], norm);
		d[2] = __ddiv_rn(d[2], norm);
		double pmax = -2., qmax = -2., P[3];
		int pok = 0;
#pragma unroll 1
		for(int a = 0; a < 4; a++) {
			patch64(Rp, base[a], P);
			double pc = scalar64(d, P);
			pmax = fmax(pmax, pc);
			if(pc > cosmax) pok = 1;
		}
#pragma unroll 1
		for(int b = 0; b < 4; b++) {
			patch64(Rq, base[b], P);
			double qc = -scalar64(d, P);
			qmax = fmax(qmax, qc);
			if(pok && qc > cosmax) res = 1;
		}
		if(o_pmax) *o_pmax = pmax;
		if(o_qmax) *o_qmax = qmax;
	}
	return res;
}

/* ------------------------------------------------------------------------------------------------ */
/* Canonical state arithmetic                                                                       */
/* ------------------------------------------------------------------------------------------------ */
/* exact FP32 -> FP64 widening by bit manipulation (integer pipe; the FP64 pipe is the scarce one);
 * equal to (double) f for every finite f */
__device__ __forceinline__ double f2d(float f) {
	uint32_t b = __float_as_uint(f);
	uint32_t e = (b >> 23) & 0xffu;
	if(e == 0u) return (double) f; /* zero or subnormal */
	uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
	return __hiloint2double((int) hi, (int) (b << 29));
}

/* FP64 -> FP32 rounded to nearest (ties away from zero) by bit manipulation; magnitudes below the FP32
 * normal range become zero. Used only for the FP32 working copies, whose error budget is ~1e-7. */
__device__ __forceinline__ float d2f(double x) {
	unsigned long long u = (unsigned long long) __double_as_longlong(x);
	uint32_t s = (uint32_t) (u >> 32) & 0x80000000u;
	u = (u & 0x7fffffffffffffffull) + 0x10000000ull;
	int e = (int) (u >> 52) - 896;
	if(e <= 0) return __uint_as_float(s);
	return __uint_as_float(s | ((uint32_t) e << 23) | ((uint32_t) (u >> 29) & 0x7fffffu));
}

/* Component c of the Hamilton product a (x) b, with a_{c^k} given as ac[k]:
 *   w' = aw bw - ax bx - ay by - az bz      x' = ax bw + aw bx - az by + ay bz
 *   y' = ay bw + az bx + aw by - ax bz      z' = az bw - ay bx + ax by + aw bz
 * i.e. c' = sum_k s(c, k) a_{c^k} b_k with the sign pattern 0x284E (one nibble per c, bit k = minus).
 * One fixed sequence of explicitly rounded operations for every c, so the lanes of a group compute
 * their components without divergence and the full product (qmul64) is bit-identical. */
__device__ __forceinline__ double qcomp64(double a0, double a1, double a2, double a3, const double *b, int c) {
	const int m = (0x284E >> (4 * c)) & 0xF;
	double v = __dmul_rn(a0, b[0]);
	v = __fma_rn((m & 2) ? -a1 : a1, b[1], v);
	v = __fma_rn((m & 4) ? -a2 : a2, b[2], v);
	v = __fma_rn((m & 8) ? -a3 : a3, b[3], v);
	return v;
}

__device__ __forceinline__ void qmul64(const double *a, const double *b, double *out) {
#pragma unroll 1
	for(int c = 0; c < 4; c++) out[c] = qcomp64(a[c], a[c ^ 1], a[c ^ 2], a[c ^ 3], b, c);
}

/* rotation matrix of q / |q| (rows), q = (w, x, y, z); the identity quaternion gives exactly I */
__device__ __forceinline__ void quatmat64(const double *q, double *Q) {
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	const double xx = __dmul_rn(x, x), yy = __dmul_rn(y, y), zz = __dmul_rn(z, z), ww = __dmul_rn(w, w);
	const double xy = __dmul_rn(x, y), xz = __dmul_rn(x, z), yz = __dmul_rn(y, z);
	const double wx = __dmul_rn(w, x), wy = __dmul_rn(w, y), wz = __dmul_rn(w, z);
	const double s = __ddiv_rn(2.0, __dadd_rn(__dadd_rn(ww, xx), __dadd_rn(yy, zz)));
	Q[0] = __dsub_rn(1.0, __dmul_rn(s, __dadd_rn(yy, zz)));
	Q[1] = __dmul_rn(s, __dsub_rn(xy, wz));
	Q[2] = __dmul_rn(s, __dadd_rn(xz, wy));
	Q[3] = __dmul_rn(s, __dadd_rn(xy, wz));
	Q[4] = __dsub_rn(1.0, __dmul_rn(s, __dadd_rn(xx, zz)));
	Q[5] = __dmul_rn(s, __dsub_rn(yz, wx));
	Q[6] = __dmul_rn(s, __dsub_rn(xz, wy));
	Q[7] = __dmul_rn(s, __dadd_rn(yz, wx));
	Q[8] = __dsub_rn(1.0, __dmul_rn(s, __dadd_rn(xx, yy)));
}

/* orientation R = R0 . Q(q) of a canonical record. With q the identity (every particle after upload or
 * orthonormalisation) the result is R0 bit for bit (up to the sign of zero entries, which no test of
 * MC_would_interact can see). */
__device__ __forceinline__ void orient64_ops(const double *R0, const double *q, double *R) {
	double Q[9];
	quatmat64(q, Q);
#pragma unroll
	for(int i = 0; i < 3; i++)
#pragma unroll
		for(int j = 0; j < 3; j++)
			R[3 * i + j] = __dadd_rn(__dadd_rn(__dmul_rn(R0[3 * i], Q[j]), __dmul_rn(R0[3 * i + 1], Q[3 + j])), __dmul_rn(R0[3 * i + 2], Q[6 + j]));
}

/* the same explicitly rounded operations out of line (the exact pair test's state) */
__device__ __noinline__ void orient64(const double *R0, const double *q, double *R) { orient64_ops(R0, q, R); }

/* Canonical state of particle slot ps as (x y z R00..R22): kind 0 = stored state, kind 1 = the candidate
 * of the current move, r + disp and q (x) dq with disp and dq the FP32 proposal widened exactly. This is
 * the engine's definition of the proposed state: FP32 tests approximate it, FP64 re-evaluations use it
 * and an accepted move stores exactly these q and r bits (k_colour's commit uses the same qcomp64). */
__device__ __noinline__ void state64(const double *__restrict__ rec_all, int ps, int kind, float4 dq, float3 disp, double *P) {
	const double *rec = rec_all + (size_t) ps * PPI_REC;
	double q[4] = { rec[PPI_Q], rec[PPI_Q + 1], rec[PPI_Q + 2], rec[PPI_Q + 3] };
	P[0] = rec[0];
	P[1] = rec[1];
	P[2] = rec[2];
	if(kind == 1) {
		const double b[4] = { f2d(dq.x), f2d(dq.y), f2d(dq.z), f2d(dq.w) };
		double qn[4];
		qmul64(q, b, qn);
		q[0] = qn[0];
		q[1] = qn[1];
		q[2] = qn[2];
		q[3] = qn[3];
		P[0] = __dadd_rn(P[0], f2d(disp.x));
		P[1] = __dadd_rn(P[1], f2d(disp.y));
		P[2] = __dadd_rn(P[2], f2d(disp.z));
	}
	orient64(rec + PPI_R0, q, P + 3);
}

/* Exact re-evaluation of one pair. p is the probing particle: kind 0 = its stored state, kind 1 = the
 * candidate of the current move (q, disp). Bit k of vol_mask scales coordinate k of both positions by
 * vol_f3[k] and uses box[k] = vol_box3[k] (the candidate box of an NPT volume move, MC.c:471-478, or of an
 * Lx move, MC.c:533-545); vol_mask = 0 leaves the box alone (the pointers are then not read). */
__device__ __noinline__ int exact_pair(const double *__restrict__ rec_all, const ppi_rparams *rp, const double *box_in, int ps, int kind, float4 q,
		float3 disp, int qs, int vol_mask, const double *vol_f3, const double *vol_box3, double *o_dist2, double *o_pmax, double *o_qmax) {
	double P[12], Qr[12], box[3];
	state64(rec_all, ps, kind, q, disp, P);
	state64(rec_all, qs, 0, q, disp, Qr);
#pragma unroll 1
	for(int k = 0; k < 3; k++) {
		box[k] = box_in[k];
		if((vol_mask >> k) & 1) {
			P[k] = __dmul_rn(P[k], vol_f3[k]);
			Qr[k] = __dmul_rn(Qr[k], vol_f3[k]);
			box[k] = vol_box3[k];
		}
	}
	return interact64(P, P + 3, Qr, Qr + 3, rp->base, box, rp->sqr_rcut, rp->cosmax, o_dist2, o_pmax, o_qmax);
}

/* Certified FP64 decision of one pair without the reference's division and square root chain.
 * The distance test is the reference's own operation sequence (MC.c:233-240), so it is bit-identical:
 * d = q - p, minimum image d - box * rint(d / box), dist2 = d . d. Only rint's argument is formed with
 * the reciprocal of the box; it can round differently from d / box only within ~1e-15 of a half
 * integer, which is checked. The patch test (MC.c:242-262) is evaluated to ~1e-15 with Newton
 * reciprocals (norm of d, norm of q); a cosine farther than DEC64_TOL from KF_cosmax is then on the same
 * side of it as the reference's FP64 value. Anything closer returns DEC64_EXACT and the caller runs the
 * bit-identical exact_pair. Returns -1 overlap, 0 no bond, 1 bond. */
#define DEC64_TOL 1e-12
#define DEC64_EXACT 2
/* what the FP32 test knew about a guard-band pair's patches: nothing certain, certainly not facing each
 * other, certainly facing each other (then only the distance is decided in FP64) */
#define PV_FULL 0
#define PV_NONE 1
#define PV_BOND 2

__device__ __forceinline__ double rcp64(double x) { /* 1 / x to ~1e-16, x > 0 */
	double r = (double) (1.0f / (float) x);
	r = r * (2.0 - x * r);
	r = r * (2.0 - x * r);
	return r;
}

__device__ __forceinline__ double rsqrt64(double x) { /* 1 / sqrt(x) to ~1e-16, x > 0 */
	double y = (double) rsqrtf((float) x);
	y = y * (1.5 - 0.5 * x * y * y);
	y = y * (1.5 - 0.5 * x * y * y);
	y = y * (1.5 - 0.5 * x * y * y);
	return y;
}

/* orientation R0 . Q(q) to ~1e-15 (the canonical value is orient64's; this is only compared with a margin) */
__device__ __forceinline__ void orient64_fast(const double *R0, const double *q, double *R) {
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	const double s = 2.0 * rcp64(w * w + x * x + y * y + z * z);
	double Q[9];
	Q[0] = 1.0 - s * (y * y + z * z);
	Q[1] = s * (x * y - w * z);
	Q[2] = s * (x * z + w * y);
	Q[3] = s * (x * y + w * z);
	Q[4] = 1.0 - s * (x * x + z * z);
	Q[5] = s * (y * z - w * x);
	Q[6] = s * (x * z - w * y);
	Q[7] = s * (y * z + w * x);
	Q[8] = 1.0 - s * (x * x + y * y);
#pragma unroll
	for(int i = 0; i < 3; i++)
#pragma unroll
		for(int j = 0; j < 3; j++) R[3 * i + j] = fma(R0[3 * i], Q[j], fma(R0[3 * i + 1], Q[3 + j], R0[3 * i + 2] * Q[6 + j]));
}

/* canonical position (bit-exact, as state64) and approximate orientation of slot ps, state kind */
__device__ __forceinline__ void state64_fast(const double *__restrict__ rec_all, int ps, int kind, float4 dq, float3 disp, double *r, double *R) {
	const double *rec = rec_all + (size_t) ps * PPI_REC;
	double q[4] = { rec[PPI_Q], rec[PPI_Q + 1], rec[PPI_Q + 2], rec[PPI_Q + 3] };
	r[0] = rec[0];
	r[1] = rec[1];
	r[2] = rec[2];
	if(kind == 1) {
		const double b[4] = { f2d(dq.x), f2d(dq.y), f2d(dq.z), f2d(dq.w) };
		double qn[4];
#pragma unroll
		for(int c = 0; c < 4; c++) qn[c] = qcomp64(q[c], q[c ^ 1], q[c ^ 2], q[c ^ 3], b, c);
#pragma unroll
		for(int c = 0; c < 4; c++) q[c] = qn[c];
		r[0] = __dadd_rn(r[0], f2d(disp.x));
		r[1] = __dadd_rn(r[1], f2d(disp.y));
		r[2] = __dadd_rn(r[2], f2d(disp.z));
	}
	double R0[9];
#pragma unroll
	for(int k = 0; k < 9; k++) R0[k] = rec[PPI_R0 + k];
	orient64_fast(R0, q, R);
}

__device__ __forceinline__ int decide64(const double *__restrict__ rec_all, const ppi_rparams &rp, const double *box_in, const double *inv_box_in, int ps, int kind, float4 dq,
		float3 disp, int qs, int vol_mask, const double *vol_f3, const double *vol_box3) {
	double rp_[3], Rp[9], rq_[3], Rq[9];
	state64_fast(rec_all, ps, kind, dq, disp, rp_, Rp);
	state64_fast(rec_all, qs, 0, dq, disp, rq_, Rq);
	double box[3] = { box_in[0], box_in[1], box_in[2] }, ib[3] = { inv_box_in[0], inv_box_in[1], inv_box_in[2] };
	if(vol_mask) {
#pragma unroll
		for(int k = 0; k < 3; k++)
			if((vol_mask >> k) & 1) {
				rp_[k] = __dmul_rn(rp_[k], vol_f3[k]);
				rq_[k] = __dmul_rn(rq_[k], vol_f3[k]);
				box[k] = vol_box3[k];
				ib[k] = rcp64(vol_box3[k]);
			}
	}
	double d[3];
#pragma unroll
	for(int k = 0; k < 3; k++) {
		d[k] = __dsub_rn(rq_[k], rp_[k]);
		const double t = d[k] * ib[k], n = rint(t);
		if(fabs(t - n) > 0.5 - 1e-9) return DEC64_EXACT; /* rint of d / box could round the other way */
		d[k] = __dsub_rn(d[k], __dmul_rn(box[k], n));
	}
	const double dist2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
	if(dist2 < 1.) return -1;
	if(!(dist2 < rp.sqr_rcut)) return 0;
	const double in = rsqrt64(dist2);
	const double u[3] = { d[0] * in, d[1] * in, d[2] * in };
	const double cmax = rp.cosmax;
	int p_yes = 0, p_unsure = 0, q_yes = 0, q_unsure = 0;
#pragma unroll
	for(int a = 0; a < 4; a++) {
		const double *b = rp.base[a];
		double c = 0.;
#pragma unroll
		for(int k = 0; k < 3; k++) c = fma(u[k], fma(Rp[3 * k], b[0], fma(Rp[3 * k + 1], b[1], Rp[3 * k + 2] * b[2])), c);
		p_yes |= c > cmax + DEC64_TOL;
		p_unsure |= fabs(c - cmax) <= DEC64_TOL;
		double e = 0.;
#pragma unroll
		for(int k = 0; k < 3; k++) e = fma(u[k], fma(Rq[3 * k], b[0], fma(Rq[3 * k + 1], b[1], Rq[3 * k + 2] * b[2])), e);
		e = -e;
		q_yes |= e > cmax + DEC64_TOL;
		q_unsure |= fabs(e - cmax) <= DEC64_TOL;
	}
	/* bond iff some patch of p and some patch of q point at each other (MC.c:249-262) */
	if(p_yes && q_yes) return 1;
	if((!p_yes && !p_unsure) || (!q_yes && !q_unsure)) return 0;
	return DEC64_EXACT;
}

/* decide64 with all 32 lanes of a warp on one pair: every lane calls it with the same arguments and gets
 * the same result. The distance test runs first on every lane (an overlap or a pair out of range needs no
 * orientation); then lanes 0..15 build p's orientation and 16..31 q's: lanes 0..3 one component each of
 * the mover's q (x) dq, lane e < 9 of each half one entry of R0 . Q(q), lanes 0..3
 * and 16..19 one patch cosine each. The values, and so the decision, are decide64's. On this GPU an FP64
 * instruction occupies the FP64 pipe as long for one lane as for 32, so spreading the ~270 FP64
 * operations of one decision over the lanes shortens the warp's wait on it several times; one guard-band
 * pair decided by a single lane was the longest chain of a colour pass. */
__device__ __forceinline__ double shfl_d(double v, int src) {
	const int lo = __shfl_sync(0xffffffffu, __double2loint(v), src), hi = __shfl_sync(0xffffffffu, __double2hiint(v), src);
	return __hiloint2double(hi, lo);
}

__device__ __forceinline__ int decide64_warp(const double *__restrict__ rec_all, const ppi_rparams &rp, const double *box_in, const double *inv_box_in, int ps, int kind,
		float4 dq, float3 disp, int qs, int vol_mask, const double *vol_f3, const double *vol_box3, int lane, int pv = 0) {
	const int half = lane >> 4, e = lane & 15;
	const double *rec = rec_all + (size_t) (half ? qs : ps) * PPI_REC;
	/* positions first: the distance test alone decides an overlap or a pair out of range */
	double r[3] = { rec[0], rec[1], rec[2] };
	if(half == 0 && kind == 1) {
		r[0] = __dadd_rn(r[0], f2d(disp.x));
		r[1] = __dadd_rn(r[1], f2d(disp.y));
		r[2] = __dadd_rn(r[2], f2d(disp.z));
	}
	double rp_[3], rq_[3], box[3] = { box_in[0], box_in[1], box_in[2] }, ib[3] = { inv_box_in[0], inv_box_in[1], inv_box_in[2] };
#pragma unroll
	for(int k = 0; k < 3; k++) {
		rp_[k] = shfl_d(r[k], 0);
		rq_[k] = shfl_d(r[k], 16);
	}
	if(vol_mask) {
#pragma unroll
		for(int k = 0; k < 3; k++)
			if((vol_mask >> k) & 1) {
				rp_[k] = __dmul_rn(rp_[k], vol_f3[k]);
				rq_[k] = __dmul_rn(rq_[k], vol_f3[k]);
				box[k] = vol_box3[k];
				ib[k] = rcp64(vol_box3[k]);
			}
	}
	double d[3];
	int exact = 0;
#pragma unroll
	for(int k = 0; k < 3; k++) {
		d[k] = __dsub_rn(rq_[k], rp_[k]);
		/* the image n = rint(d / box): from an FP32 estimate where it is certain (|tf - t| <= 3 2^-24 |t| < 0.02,
		 * so a tf within 0.25 of an integer rounds like t, and t is not near a half), else in FP64 */
		const float tf = d2f(d[k]) * d2f(ib[k]), nf = rintf(tf);
		if(fabsf(tf - nf) < 0.25f && fabsf(tf) < 1e5f) {
			if(nf != 0.f) d[k] = __dsub_rn(d[k], __dmul_rn(box[k], f2d(nf)));
		}
		else {
			const double t = d[k] * ib[k], n = rint(t);
			if(fabs(t - n) > 0.5 - 1e-9) exact = 1; /* rint of d / box could round the other way */
			d[k] = __dsub_rn(d[k], __dmul_rn(box[k], n));
		}
	}
	if(exact) return DEC64_EXACT;
	const double dist2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
	if(dist2 < 1.) return -1;
	if(!(dist2 < rp.sqr_rcut)) return 0;
	if(pv != PV_FULL) return pv == PV_BOND; /* the FP32 patch test was certain: only the distance was in doubt */
	/* this half's quaternion (state64_fast): lane c < 4 of half 0 forms component c of q (x) dq */
	double q[4] = { rec[PPI_Q], rec[PPI_Q + 1], rec[PPI_Q + 2], rec[PPI_Q + 3] };
	if(kind == 1) {
		const double b[4] = { f2d(dq.x), f2d(dq.y), f2d(dq.z), f2d(dq.w) };
		const int c = e & 3;
		const double qc = qcomp64(q[c], q[c ^ 1], q[c ^ 2], q[c ^ 3], b, c);
		double qn[4];
#pragma unroll
		for(int k = 0; k < 4; k++) qn[k] = shfl_d(qc, k);
		if(half == 0)
#pragma unroll
			for(int k = 0; k < 4; k++) q[k] = qn[k];
	}
	/* entry (i, j) = e of R = R0 . Q(q), orient64_fast's operations */
	double Rij;
	{
		const double w = q[0], x = q[1], y = q[2], z = q[3];
		const double sc = 2.0 * rcp64(w * w + x * x + y * y + z * z);
		const double Q[9] = { 1.0 - sc * (y * y + z * z), sc * (x * y - w * z), sc * (x * z + w * y), sc * (x * y + w * z), 1.0 - sc * (x * x + z * z),
			sc * (y * z - w * x), sc * (x * z - w * y), sc * (y * z + w * x), 1.0 - sc * (x * x + y * y) };
		const int i = e < 9 ? e / 3 : 0, j = e < 9 ? e % 3 : 0;
		const double *R0 = rec + PPI_R0;
		Rij = fma(R0[3 * i], Q[j], fma(R0[3 * i + 1], Q[3 + j], R0[3 * i + 2] * Q[6 + j]));
	}
	/* the halves' orientations to every lane that forms a patch (all lanes take part in the shuffles) */
	double Rm[9];
#pragma unroll
	for(int k = 0; k < 9; k++) Rm[k] = shfl_d(Rij, (half << 4) + k);
	const double in = rsqrt64(dist2);
	const double u[3] = { d[0] * in, d[1] * in, d[2] * in };
	const double cmax = rp.cosmax;
	/* lane e < 4 of each half: patch e of its particle; q's cosines are -(u . patch) */
	int yes = 0, unsure = 0;
	if(e < 4) {
		const double *b = rp.base[e];
		double c = 0.;
#pragma unroll
		for(int k = 0; k < 3; k++) c = fma(u[k], fma(Rm[3 * k], b[0], fma(Rm[3 * k + 1], b[1], Rm[3 * k + 2] * b[2])), c);
		if(half) c = -c;
		yes = c > cmax + DEC64_TOL;
		unsure = fabs(c - cmax) <= DEC64_TOL;
	}
	const unsigned by = __ballot_sync(0xffffffffu, yes), bu = __ballot_sync(0xffffffffu, unsure);
	const int p_yes = (by & 0xfu) != 0, q_yes = (by & 0xf0000u) != 0, p_unsure = (bu & 0xfu) != 0, q_unsure = (bu & 0xf0000u) != 0;
	/* bond iff some patch of p and some patch of q point at each other (MC.c:249-262) */
	if(p_yes && q_yes) return 1;
	if((!p_yes && !p_unsure) || (!q_yes && !q_unsure)) return 0;
	return DEC64_EXACT;
}

/* ------------------------------------------------------------------------------------------------ */
/* FP32 classification with guard band                                                              */
/* ------------------------------------------------------------------------------------------------ */
#define CL_OVER 0
#define CL_NONE 1
#define CL_BOND 2
#define CL_UNSURE 3

struct PairF {
	float r2, pmax, qmax;
};

/* d = q - p (cell-local frame), cp = p's orientation columns, cq = q's */
__device__ __forceinline__ int classify(float dx, float dy, float dz, const float *cp, const float *cq, float sqr_rcut, float cosmax, float base, float eps,
		PairF *diag) {
	float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
	if(diag) {
		diag->r2 = r2;
		diag->pmax = diag->qmax = -2.f;
	}
	if(r2 < 1.f - eps) return CL_OVER;
	if(r2 <= 1.f + eps) return CL_UNSURE;
	if(r2 >= sqr_rcut + eps) return CL_NONE;
	float inv = rsqrtf(r2) * base;
	float a0 = fmaf(dx, cp[0], fmaf(dy, cp[1], dz * cp[2]));
	float a1 = fmaf(dx, cp[3], fmaf(dy, cp[4], dz * cp[5]));
	float a2 = fmaf(dx, cp[6], fmaf(dy, cp[7], dz * cp[8]));
	/* patch i of p: base_i = b * s_i with s = (-,-,+), (+,-,-), (+,+,+), (-,+,-) (system.c:24-27) */
	float pm = fmaxf(fmaxf(-a0 - a1 + a2, a0 - a1 - a2), fmaxf(a0 + a1 + a2, -a0 + a1 - a2)) * inv;
	float b0 = fmaf(dx, cq[0], fmaf(dy, cq[1], dz * cq[2]));
	float b1 = fmaf(dx, cq[3], fmaf(dy, cq[4], dz * cq[5]));
	float b2 = fmaf(dx, cq[6], fmaf(dy, cq[7], dz * cq[8]));
	/* q's cosines are -(d . patch) (MC.c:254) */
	float qm = fmaxf(fmaxf(b0 + b1 - b2, -b0 + b1 + b2), fmaxf(-b0 - b1 - b2, b0 - b1 + b2)) * inv;
	if(diag) {
		diag->pmax = pm;
		diag->qmax = qm;
	}
	int unsure = (r2 > sqr_rcut - eps);
	if(!unsure) {
		if(pm < cosmax - eps || qm < cosmax - eps) return CL_NONE;
		if(pm > cosmax + eps && qm > cosmax + eps) return CL_BOND;
	}
	return CL_UNSURE;
}

/* classify with the patch verdict of a guard-band pair: the patches are tested in FP32 for every pair
 * within r_cut^2 + eps, also inside the contact band. A pair near r_cut whose patches certainly do not face
 * each other is decided here (no bond, and r^2 > 1 + eps rules out an overlap); a guard-band pair whose
 * patch verdict is certain reports it in *pv, so that the FP64 test only decides the distance. The
 * patch verdict uses the same bounds as classify's (its error bound does not depend on r^2 >= 1 - eps). */
__device__ __forceinline__ int classify_pv(float dx, float dy, float dz, const float *cp, const float *cq, float sqr_rcut, float cosmax, float base, float eps, int *pv) {
	const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
	*pv = PV_FULL;
	if(r2 < 1.f - eps) return CL_OVER;
	if(r2 >= sqr_rcut + eps) return CL_NONE;
	const float inv = rsqrtf(r2) * base;
	const float a0 = fmaf(dx, cp[0], fmaf(dy, cp[1], dz * cp[2]));
	const float a1 = fmaf(dx, cp[3], fmaf(dy, cp[4], dz * cp[5]));
	const float a2 = fmaf(dx, cp[6], fmaf(dy, cp[7], dz * cp[8]));
	const float pm = fmaxf(fmaxf(-a0 - a1 + a2, a0 - a1 - a2), fmaxf(a0 + a1 + a2, -a0 + a1 - a2)) * inv;
	const float b0 = fmaf(dx, cq[0], fmaf(dy, cq[1], dz * cq[2]));
	const float b1 = fmaf(dx, cq[3], fmaf(dy, cq[4], dz * cq[5]));
	const float b2 = fmaf(dx, cq[6], fmaf(dy, cq[7], dz * cq[8]));
	const float qm = fmaxf(fmaxf(b0 + b1 - b2, -b0 + b1 + b2), fmaxf(-b0 - b1 - b2, b0 - b1 + b2)) * inv;
	const bool pnone = pm < cosmax - eps || qm < cosmax - eps, pbond = pm > cosmax + eps && qm > cosmax + eps;
	const bool near1 = r2 <= 1.f + eps, nearc = r2 > sqr_rcut - eps;
	if(!near1 && !nearc) return pnone ? CL_NONE : (pbond ? CL_BOND : CL_UNSURE);
	if(!near1 && pnone) return CL_NONE;
	*pv = pnone ? PV_NONE : (pbond ? PV_BOND : PV_FULL);
	return CL_UNSURE;
}

__device__ __forceinline__ void atomicMaxFloatBits(unsigned int *addr, float v) {
	if(v > 0.f) atomicMax(addr, __float_as_uint(v)); /* positive floats order like their bit patterns */
}

/* audit: compare an FP32 decision, and the certified FP64 decision, with the exact one */
__device__ __noinline__ void audit_pair(const double *rec_all, const ppi_rparams *rp, ppi_rstate *rs, const double *box, const double *inv_box, int ps, int kind,
		float4 q, float3 disp, int qs, int vol_mask, const double *vol_f3, const double *vol_box3, int cl, PairF f) {
	double d2, pm = -2., qm = -2.;
	int ex = exact_pair(rec_all, rp, box, ps, kind, q, disp, qs, vol_mask, vol_f3, vol_box3, &d2, &pm, &qm);
	int exc = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
	if(cl != CL_UNSURE && cl != exc) atomicAdd(&rs->mismatches, 1ull);
	const int dc = decide64(rec_all, *rp, box, inv_box, ps, kind, q, disp, qs, vol_mask, vol_f3, vol_box3);
	if(dc != DEC64_EXACT && dc != ex) atomicAdd(&rs->mismatches, 1ull);
	if(d2 < (double) rp->sqr_rcut + 0.5) atomicMaxFloatBits(&rs->max_err_r2_bits, (float) fabs((double) f.r2 - d2));
	if(pm > -1.5 && f.pmax > -1.5f) {
		atomicMaxFloatBits(&rs->max_err_cos_bits, (float) fabs((double) f.pmax - pm));
		atomicMaxFloatBits(&rs->max_err_cos_bits, (float) fabs((double) f.qmax - qm));
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* cell grid, counting sort into cell order, colour lists                                           */
/* ------------------------------------------------------------------------------------------------ */
#define TAG_GRID 4u
#define TAG_VOL 5u
#define TAG_COLOUR 6u

/* one warp per replica, lane a < 3 for axis a (each axis' FP64 divisions on its own lane) */
__global__ void k_grid(ppi_dev d, long long epoch) {
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t == 0 && d.vp_count) { /* the counters of the list build that follows the sort (ppi_nlist) */
		d.vp_count[0] = 0;
		d.vp_count[1] = 0;
	}
	const int r = t >> 5, lane = t & 31;
	if(r >= d.nrep) return; /* the whole warp */
	epoch = ctr_index(epoch, epoch < 0 ? d.ctr->epoch : 0);
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	ppi_grid *g = d.grid + r;
	const U4 u = rng(rp, epoch, r, TAG_GRID, 0, 0);
	const int a = lane < 3 ? lane : 0;
	int err = 0;
	int k = (int) floor(rs->box[a] / rp.w_min);
	if(k > PPI_MAX_AXIS_CELLS) k = PPI_MAX_AXIS_CELLS;
	k &= ~1; /* even: the 2x2x2 checkerboard needs alternating colours across the periodic boundary */
	if(k < 4) {
		err = 1;
		k = 4;
	}
	int n[3] = { __shfl_sync(0xffffffffu, k, 0), __shfl_sync(0xffffffffu, k, 1), __shfl_sync(0xffffffffu, k, 2) };
	err = __shfl_sync(0xffffffffu, err, 0) | __shfl_sync(0xffffffffu, err, 1) | __shfl_sync(0xffffffffu, err, 2);
	/* stay inside the reserved cell capacity by coarsening the longest axis (coarser cells stay valid) */
	while((long long) n[0] * n[1] * n[2] > rp.cell_cap) {
		int ax = (n[0] >= n[1] && n[0] >= n[2]) ? 0 : (n[1] >= n[2] ? 1 : 2);
		if(n[ax] <= 4) {
			err = 1;
			break;
		}
		n[ax] -= 2;
	}
	if(lane < 3) {
		const int na = lane == 0 ? n[0] : (lane == 1 ? n[1] : n[2]);
		const float us = u01(lane == 0 ? u.x : (lane == 1 ? u.y : u.z));
		const double w = rs->box[a] / na;
		g->n[a] = na;
		g->w[a] = w;
		g->wf[a] = (float) w;
		g->shift[a] = (double) us * w;
		g->shiftf[a] = (float) g->shift[a];
		g->inv_w[a] = 1.0 / w;
		g->inv_L[a] = 1.0 / rs->box[a];
		g->inv_wf[a] = (float) g->inv_w[a];
		g->inv_Lf[a] = (float) g->inv_L[a];
		g->Lf[a] = (float) rs->box[a];
	}
	if(lane == 0) {
		g->ncells = n[0] * n[1] * n[2];
		if(err) rs->error = PPI_E_GRID;
	}
}

/* d2f truncated toward zero (the guesses below only need ~1e-7) */
__device__ __forceinline__ float d2f_trunc(double x) {
	const unsigned long long u = (unsigned long long) __double_as_longlong(x);
	const int e = (int) ((u >> 52) & 0x7ff) - 896;
	if(e <= 0) return 0.f;
	return __uint_as_float(((uint32_t) (u >> 32) & 0x80000000u) | ((uint32_t) e << 23) | ((uint32_t) (u >> 29) & 0x7fffffu));
}

/* cell of a slot in the current grid and its cell-local coordinates (FP32). The FP64 pipe is the scarce
 * resource on this GPU, so per axis the periodic image and the cell are first estimated in FP32: where
 * the estimate lies farther than its error bound m from the box and cell boundaries, both are certain and
 * the FP64 work is three explicitly rounded operations (image, grid origin, cell origin). Otherwise the
 * image and the cell are found by the careful path: FP32 guesses of both, each checked against the FP64
 * value and corrected. |estimate - exact| <= 2^-23 |x| + 2^-24 (|k| + 3) L, and m is ~8x that. */
__global__ void k_assign(ppi_dev d, float4 *tmp) {
	grid_dep_wait(); /* chained by programmatic dependent launch (ppi_resort) */
	grid_dep_release();
	int s = blockIdx.x * blockDim.x + threadIdx.x;
	if(s >= d.ntot) return;
	const int r = d.rep[s];
	const ppi_grid &g = d.grid[r];
	const double *x = d.rec + (size_t) s * PPI_REC;
	const double2 x01 = *(const double2 *) x;
	const double xs[3] = { x01.x, x01.y, x[2] };
	int c[3];
	float l[3];
#pragma unroll
	for(int a = 0; a < 3; a++) {
		const double L = d.rs[r].box[a], w = g.w[a];
		const int n = g.n[a];
		const float Lf = g.Lf[a], wf = g.wf[a];
		/* periodic image: x - k L in [0, L) */
		const float xf = d2f_trunc(xs[a]);
		const float kf = floorf(xf * g.inv_Lf[a]);
		const float yg = fmaf(-kf, Lf, xf) - g.shiftf[a];
		const float cg = floorf(yg * g.inv_wf[a]);
		const float lg = fmaf(-cg, wf, yg);
		const float m = 1e-6f * (fabsf(xf) + (fabsf(kf) + 3.f) * Lf);
		int ci;
		float lf;
		if(__builtin_expect(yg >= m && yg < Lf - m && lg >= m && lg < wf - m && cg < (float) n, 1)) {
			ci = (int) cg;
			/* k = 0 (the particle's own image, the usual case): fma(-0, L, x) = x */
			const double y = __dadd_rn(kf == 0.f ? xs[a] : __fma_rn(-f2d(kf), L, xs[a]), -g.shift[a]);
			lf = d2f(__fma_rn(-f2d(cg), w, y));
		}
		else {
			double y = __dadd_rn(__fma_rn(-f2d(kf), L, xs[a]), -g.shift[a]);
			float yf = d2f_trunc(y);
			if(yf < 0.f) y += L;
			else if(yf >= Lf) y -= L;
			yf = d2f_trunc(y);
			if(yf < 0.f) y += L; /* a guess of k off by one in both steps: one more image */
			else if(yf >= Lf) y -= L;
			ci = (int) (d2f_trunc(y) * g.inv_wf[a]);
			ci = ci < 0 ? 0 : (ci > n - 1 ? n - 1 : ci);
			lf = d2f(__fma_rn(-f2d((float) ci), w, y));
			if(lf < 0.f && ci > 0) {
				--ci;
				lf = d2f(__fma_rn(-f2d((float) ci), w, y));
			}
			else if(lf >= wf && ci < n - 1) {
				++ci;
				lf = d2f(__fma_rn(-f2d((float) ci), w, y));
			}
		}
		c[a] = ci;
		l[a] = lf;
	}
	const int gc = d.rp[r].cell_base + (c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
	d.cellof[s] = gc;
	/* .w = the particle's rank among its cell's arrivals (the scatter's offset in the cell; k_cellfin
	 * then orders each cell by particle id) */
	tmp[s] = make_float4(l[0], l[1], l[2], __int_as_float(atomicAdd(d.cell_count + gc, 1)));
}

#define SCAN_B 1024
/* inclusive scan of v over the CTA (SCAN_B threads): warp shuffles, then the warps' totals */
__device__ __forceinline__ int block_scan_incl(int v, int *ws) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		const int y = __shfl_up_sync(0xffffffffu, v, o);
		if(lane >= o) v += y;
	}
	if(lane == 31) ws[warp] = v;
	__syncthreads();
	if(warp == 0) {
		int t = ws[lane];
#pragma unroll
		for(int o = 1; o < 32; o <<= 1) {
			const int y = __shfl_up_sync(0xffffffffu, t, o);
			if(lane >= o) t += y;
		}
		ws[lane] = t;
	}
	__syncthreads();
	if(warp > 0) v += ws[warp - 1];
	return v;
}

#define SCAN_T 4                    /* cells per thread of the scan */
#define SCAN_TILE (SCAN_B * SCAN_T) /* cells per CTA */
#define SCAN_SHIFT 12               /* log2(SCAN_TILE) */

/* Cell starts in one launch: every CTA scans its tile of SCAN_TILE cell counts (the tile-local exclusive
 * prefix goes to part) and publishes the tile's total in aux; the CTA that finishes last (a ticket counter,
 * zeroed before the sort) turns aux into the tiles' exclusive offsets and writes the grand total to
 * *total_out, the end of the last cell. The start of cell c is then part[c] + aux[c >> SCAN_SHIFT]:
 * k_scatter reads it so, and k_cellfin writes it to cell_start for every later reader. */
__global__ void __launch_bounds__(SCAN_B) k_scan(const int *in, int *part, int *aux, int *ticket, int *total_out, int n) {
	grid_dep_wait(); /* chained by programmatic dependent launch (ppi_resort) */
	grid_dep_release();
	__shared__ int ws[SCAN_B / 32];
	__shared__ int s_last;
	const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_T;
	int v[SCAN_T];
	const bool full = base + SCAN_T <= n;
	if(full) {
		const int4 q = *(const int4 *) (in + base);
		v[0] = q.x;
		v[1] = q.y;
		v[2] = q.z;
		v[3] = q.w;
	}
	else {
#pragma unroll
		for(int k = 0; k < SCAN_T; k++) v[k] = base + k < n ? in[base + k] : 0;
	}
	const int tsum = v[0] + v[1] + v[2] + v[3];
	const int x = block_scan_incl(tsum, ws);
	int p[SCAN_T];
	p[0] = x - tsum;
#pragma unroll
	for(int k = 1; k < SCAN_T; k++) p[k] = p[k - 1] + v[k - 1];
	if(full) *(int4 *) (part + base) = make_int4(p[0], p[1], p[2], p[3]);
	else {
#pragma unroll
		for(int k = 0; k < SCAN_T; k++)
			if(base + k < n) part[base + k] = p[k];
	}
	if(threadIdx.x == SCAN_B - 1) {
		aux[blockIdx.x] = x;
		__threadfence(); /* the tile total is visible before the ticket is taken */
		s_last = atomicAdd(ticket, 1) == (int) gridDim.x - 1;
	}
	__syncthreads();
	if(!s_last) return;
	__threadfence(); /* every other tile's total was published before its ticket */
	int carry = 0;
	const int nblocks = gridDim.x;
	for(int b0 = 0; b0 < nblocks; b0 += SCAN_B) {
		const int i = b0 + threadIdx.x;
		const int t = (i < nblocks) ? __ldcg(aux + i) : 0;
		const int y = block_scan_incl(t, ws);
		if(i < nblocks) aux[i] = carry + y - t;
		carry += ws[SCAN_B / 32 - 1]; /* the chunk's total */
		__syncthreads();
	}
	if(threadIdx.x == 0) *total_out = carry;
}

/* FP32 working record of slot s at sorted position pos: cell-local position from k_assign, orientation
 * columns of R0 . Q(q) evaluated in FP32 (error ~1e-7, far inside the guard band) */
__global__ void k_scatter(ppi_dev d, const float4 *tmp) {
	grid_dep_wait(); /* chained by programmatic dependent launch (ppi_resort) */
	grid_dep_release();
	int s = blockIdx.x * blockDim.x + threadIdx.x;
	if(s >= d.ntot) return;
	int gc = d.cellof[s];
	float4 a = tmp[s];
	int pos = d.cell_part[gc] + d.scan_aux[gc >> SCAN_SHIFT] + __float_as_int(a.w); /* cell start (k_scan) + arrival rank */
	const double *rec = d.rec + (size_t) s * PPI_REC;
	{ /* .w = the cell's x index (neighbour offsets in the colour pass) */
		const int r = d.rep[s];
		a.w = __int_as_float((gc - d.rp[r].cell_base) % d.grid[r].n[0]);
		if(d.srep) d.srep[pos] = r;
	}
	static_assert(PPI_Q == 3 && PPI_R0 == 7 && PPI_REC == 16, "record layout");
	/* doubles 2..15 of the 128 B record in seven 16 B loads: q = 3..6, R0 = 7..15 */
	const double2 *r2 = (const double2 *) rec;
	const double2 v1 = r2[1], v2 = r2[2], v3 = r2[3], v4 = r2[4], v5 = r2[5], v6 = r2[6], v7 = r2[7];
	const float R0[9] = { d2f(v3.y), d2f(v4.x), d2f(v4.y), d2f(v5.x), d2f(v5.y), d2f(v6.x), d2f(v6.y), d2f(v7.x), d2f(v7.y) };
	float Q[9];
	const float w = d2f(v1.y), x = d2f(v2.x), y = d2f(v2.y), z = d2f(v3.x);
	const float sc = 2.f / (w * w + x * x + y * y + z * z);
	Q[0] = 1.f - sc * (y * y + z * z);
	Q[1] = sc * (x * y - w * z);
	Q[2] = sc * (x * z + w * y);
	Q[3] = sc * (x * y + w * z);
	Q[4] = 1.f - sc * (x * x + z * z);
	Q[5] = sc * (y * z - w * x);
	Q[6] = sc * (x * z - w * y);
	Q[7] = sc * (y * z + w * x);
	Q[8] = 1.f - sc * (x * x + y * y);
	float c[9]; /* c[3 j + i] = R_ij */
#pragma unroll
	for(int i = 0; i < 3; i++)
#pragma unroll
		for(int j = 0; j < 3; j++) c[3 * j + i] = fmaf(R0[3 * i], Q[j], fmaf(R0[3 * i + 1], Q[3 + j], R0[3 * i + 2] * Q[6 + j]));
	d.spos[pos] = a;
	float4 *o = d.sori + 3 * (size_t) pos;
	o[0] = make_float4(c[0], c[1], c[2], c[3]);
	o[1] = make_float4(c[4], c[5], c[6], c[7]);
	o[2] = make_float4(c[8], __int_as_float(d.id[s]), __int_as_float(gc), __int_as_float(s));
}

/* per cell: deterministic order (ascending particle id); the colour lists of non-empty cells, built per
 * CTA (ballot ranks inside each warp, one global atomic per colour and CTA). A list entry carries what an
 * attempt needs first: (global cell, first sorted position, particle count, replica). */
#define CELLFIN_B 256
__global__ void __launch_bounds__(CELLFIN_B) k_cellfin(ppi_dev d) {
	grid_dep_wait(); /* chained by programmatic dependent launch (ppi_resort) */
	grid_dep_release();
	__shared__ int s_cnt[CELLFIN_B / 32][8];
	__shared__ int s_base[8];
	const int gc = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int col = -1, a_out = 0, b_out = 0, rep_out = 0;
	if(gc < d.total_cells) {
		/* the cell's start from k_scan's tile prefix and tile offset, written out for every later reader
		 * (the end of the last cell, cell_start[total_cells], was written by k_scan) */
		const int a = d.cell_part[gc] + d.scan_aux[gc >> SCAN_SHIFT];
		const int b = gc + 1 < d.total_cells ? d.cell_part[gc + 1] + d.scan_aux[(gc + 1) >> SCAN_SHIFT] : d.cell_start[gc + 1];
		d.cell_start[gc] = a;
		const int r = d.cell_rep[gc];
		const ppi_grid &g = d.grid[r];
		const int local = gc - d.rp[r].cell_base;
		if(local < g.ncells) {
			a_out = a;
			b_out = b;
			rep_out = r;
			if(b > a) {
				const int cx = local % g.n[0], cy = (local / g.n[0]) % g.n[1], cz = local / (g.n[0] * g.n[1]);
				col = (cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2);
			}
		}
	}
	int rank = 0;
#pragma unroll
	for(int c = 0; c < 8; c++) {
		const unsigned m = __ballot_sync(0xffffffffu, col == c);
		if(col == c) rank = __popc(m & ((1u << lane) - 1u));
		if(lane == 0) s_cnt[warp][c] = __popc(m);
	}
	__syncthreads();
	if(threadIdx.x < 8) {
		const int c = threadIdx.x;
		int tot = 0;
		for(int w = 0; w < CELLFIN_B / 32; w++) {
			const int v = s_cnt[w][c];
			s_cnt[w][c] = tot;
			tot += v;
		}
		s_base[c] = tot ? atomicAdd(d.ccount + c, tot) : 0;
	}
	__syncthreads();
	if(col >= 0) {
		const int idx = s_base[col] + s_cnt[warp][col] + rank;
		if(idx < d.clist_cap) d.clist[(size_t) col * d.clist_cap + idx] = make_int4(gc, a_out, b_out - a_out, rep_out);
	}
	/* the cell's records by ascending id (after the CTA's barriers: the other warps do not wait for it) */
	if(b_out - a_out > 1) {
		const int a = a_out, b = b_out;
		float4 *P = d.spos, *O = d.sori;
		for(int i = a + 1; i < b; i++) {
			const float4 x0 = P[i], x1 = O[3 * i], x2 = O[3 * i + 1], x3 = O[3 * i + 2];
			const int key = __float_as_int(x3.y);
			int j = i - 1;
			while(j >= a && __float_as_int(O[3 * j + 2].y) > key) {
				P[j + 1] = P[j];
				O[3 * (j + 1)] = O[3 * j];
				O[3 * (j + 1) + 1] = O[3 * j + 1];
				O[3 * (j + 1) + 2] = O[3 * j + 2];
				j--;
			}
			P[j + 1] = x0;
			O[3 * (j + 1)] = x1;
			O[3 * (j + 1) + 1] = x2;
			O[3 * (j + 1) + 2] = x3;
		}
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* one checkerboard colour: one attempt per non-empty cell of that colour                           */
/* ------------------------------------------------------------------------------------------------ */
/* per-thread counters of one launch; reduced per CTA when the CTA serves one replica (the usual case),
 * otherwise flushed per thread */
struct Acc {
	int r;
	unsigned tries, acc, pairs, fallbacks;
	int dbonds;
};

__device__ __forceinline__ void flush_thread(const ppi_dev &d, Acc &A) {
	if(A.r < 0) return;
	ppi_rstate *rs = d.rs + A.r;
	if(A.tries) atomicAdd(&rs->tries[0], (unsigned long long) A.tries);
	if(A.acc) atomicAdd(&rs->accepted[0], (unsigned long long) A.acc);
	if(A.pairs) atomicAdd(&rs->pairs, (unsigned long long) A.pairs);
	if(A.fallbacks) atomicAdd(&rs->fallbacks, (unsigned long long) A.fallbacks);
	if(A.dbonds) atomicAdd((unsigned long long *) &rs->bonds, (unsigned long long) (long long) A.dbonds);
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
}

/* block-wide flush: every thread of the CTA must call it */
__device__ __forceinline__ void flush_block(const ppi_dev &d, Acc &A) {
	__shared__ int s_rep, s_mixed;
	__shared__ unsigned s_v[4];
	__shared__ int s_db;
	if(threadIdx.x == 0) {
		s_rep = -1;
		s_mixed = 0;
		s_v[0] = s_v[1] = s_v[2] = s_v[3] = 0;
		s_db = 0;
	}
	__syncthreads();
	if(A.r >= 0) {
		int old = atomicCAS(&s_rep, -1, A.r);
		if(old != -1 && old != A.r) s_mixed = 1;
	}
	__syncthreads();
	if(s_mixed) {
		flush_thread(d, A);
		return;
	}
	unsigned t = __reduce_add_sync(0xffffffffu, A.tries), ac = __reduce_add_sync(0xffffffffu, A.acc);
	unsigned p = __reduce_add_sync(0xffffffffu, A.pairs), f = __reduce_add_sync(0xffffffffu, A.fallbacks);
	int db = __reduce_add_sync(0xffffffffu, A.dbonds);
	if((threadIdx.x & 31) == 0 && (t | p)) {
		atomicAdd(&s_v[0], t);
		atomicAdd(&s_v[1], ac);
		atomicAdd(&s_v[2], p);
		atomicAdd(&s_v[3], f);
		atomicAdd(&s_db, db);
	}
	__syncthreads();
	if(threadIdx.x == 0 && s_rep >= 0 && (s_v[0] | s_v[2])) {
		ppi_rstate *rs = d.rs + s_rep;
		if(s_v[0]) atomicAdd(&rs->tries[0], (unsigned long long) s_v[0]);
		if(s_v[1]) atomicAdd(&rs->accepted[0], (unsigned long long) s_v[1]);
		if(s_v[2]) atomicAdd(&rs->pairs, (unsigned long long) s_v[2]);
		if(s_v[3]) atomicAdd(&rs->fallbacks, (unsigned long long) s_v[3]);
		if(s_db) atomicAdd((unsigned long long *) &rs->bonds, (unsigned long long) (long long) s_db);
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* one checkerboard colour: one attempt per non-empty cell of that colour, 64 attempts per warp      */
/* ------------------------------------------------------------------------------------------------ */
/* Kernel modes of the colour and energy passes:
 *   MODE_FAST  pair tests in FP32; a pair inside the guard band is re-evaluated exactly (FP64, out of
 *              line, rare)
 *   MODE_AUDIT every pair additionally re-evaluated in FP64 and compared (test mode) */
#define MODE_FAST 0
#define MODE_AUDIT 2
#ifndef PPI_FAST_MIN_BLOCKS
#define PPI_FAST_MIN_BLOCKS 6 /* resident 128-thread CTAs per SM the energy kernels are compiled for */
#endif
#define TILE_WARPS 3 /* warps per CTA of the colour kernel (shared memory: ~12 KB per warp) */
#ifndef PPI_TILE_MIN_BLOCKS
#define PPI_TILE_MIN_BLOCKS 5 /* resident CTAs per SM of the colour kernel (measured: 5 beats 6, 128 registers) */
#endif
#ifndef PPI_VOL_MIN_BLOCKS
#define PPI_VOL_MIN_BLOCKS 6 /* resident CTAs per SM of the candidate-box energy kernel */
#endif

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

/* the FP32 decision for one pair and one state of p, made exact in the guard band */
template <int MODE>
__device__ __forceinline__ int pair_state(const double *rec, const ppi_rparams &rp, ppi_rstate *rs, const double *inv_box, int pslot, int kind, float4 q, float3 disp,
		int qslot, float dx, float dy, float dz, const float *cp, const float *cq, float sqr_rcut, float cosmax, float basef, float eps, int vol_mask,
		const double *vol_f3, const double *vol_box3, unsigned &fallbacks) {
	PairF f;
	int cl = classify(dx, dy, dz, cp, cq, sqr_rcut, cosmax, basef, eps, MODE == MODE_AUDIT ? &f : nullptr);
	if(MODE == MODE_AUDIT) audit_pair(rec, &rp, rs, rs->box, inv_box, pslot, kind, q, disp, qslot, vol_mask, vol_f3, vol_box3, cl, f);
	if(cl == CL_UNSURE) {
		fallbacks++;
		int ex = decide64(rec, rp, rs->box, inv_box, pslot, kind, q, disp, qslot, vol_mask, vol_f3, vol_box3);
		if(ex == DEC64_EXACT) ex = exact_pair(rec, &rp, rs->box, pslot, kind, q, disp, qslot, vol_mask, vol_f3, vol_box3, nullptr, nullptr, nullptr);
		cl = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
	}
	return cl;
}


/* Colour pass design. A warp takes TA = 64 list entries at a time; lane l owns attempts l and l + 32
 * for the per-attempt work (draws, proposal, decision, commit). The neighbour pairs of the 64 attempts
 * are flattened, one neighbour plane (dz) at a time, into a shared pair list (a warp scan of the lanes'
 * plane lengths gives each attempt its slice), and the lanes then walk that list 32 pairs per step,
 * PSTEP steps' candidate loads in flight together: every lane executes the same instructions on its own
 * pair, so the warp does not serialise the attempts' differently sized neighbourhoods. Pairs within the
 * bonding range are compacted (ballot) into a second list whose steps run the patch tests.
 * An attempt with a pair inside the guard band (or whose pairs do not fit the list) is not decided in
 * the loop: it is deferred to the end of the warp's share of the colour, where it is re-run on its own
 * with the FP64 fallback (attempt_exact). Same-colour attempts never see each other, so the order does
 * not matter; keeping the out-of-line FP64 code out of the loop keeps the loop free of spills. */
#define TA 64          /* attempts per warp and iteration (2 per lane) */
#define TILE_PCAP 768  /* pair list capacity per neighbour plane */
#define TILE_CCAP 128  /* close-pair list capacity, >= 32 * PSTEP (flushed before it can overflow) */
#define TILE_DCAP 16   /* deferred attempts a warp keeps in shared memory (more: flags in global memory) */
#define TILE_UCAP 32   /* guard-band pairs per iteration resolved in place (more: the attempt is deferred) */
#ifndef PSTEP
#define PSTEP 4        /* pair steps whose candidate loads are issued together */
#endif
#define TILE_OFF_MAX (1 << 21) /* |candidate - mover| sorted-position distance that a packed entry holds */
#define TF_OVER 1      /* the candidate state overlaps: rejected */
#define TF_DEFER 2     /* decided at the end, exactly (guard-band pair, or pairs beyond the list) */
#define TF_CLOSED 4    /* no attempt (empty slot or move out of the cell) */

struct __align__(16) TileSmem {
	float4 pos[TA];   /* old cell-local position, .w = cell x index */
	float4 md[TA];    /* displacement, .w = mover slot */
	float4 wv[TA];    /* cell edges (wx, wy, wz), .w = number of x cells */
	float4 qr[TA];    /* proposed rotation quaternion */
	float cpo[9][TA]; /* mover's old orientation columns */
	float2 lim[TA];   /* (1 - eps, r_cut^2 + eps): certain overlap below, certainly unbonded above */
	int mi[TA];       /* mover sorted position */
	int rep[TA];      /* replica */
	int cc[TA];       /* mover cell coordinates cx | cy << 10 | cz << 20 */
	int flag[TA], bo[TA], bn[TA];
	int pbuf[TILE_PCAP]; /* (candidate - mover) << 10 | attempt << 4 | row */
	int cbuf[TILE_CCAP]; /* same packing, pairs within the bonding range */
	int dl[TILE_DCAP];   /* list indices of deferred attempts */
	int2 uns[TILE_UCAP]; /* guard-band pairs of this iteration: (sorted position, patch verdict << 7 | attempt << 1 | kind) */
	int nc, nd, dov, nu;
};

/* the proposal of one attempt: particle, displacement, rotation (MC_move_rototranslate, MC.c:311-340) */
struct Proposal {
	int i, r, local, pslot, inside;
	float4 po, q;
	float3 disp;
	float cpo[9];
};

/* the attempt's Philox draws (particle + displacement, rotation; acceptance only when needed) and its mover */
__device__ __forceinline__ void propose_draws(const ppi_dev &d, const int4 ent, long long round, Proposal &P, U4 &r1, U4 &r2) {
	P.r = ent.w;
	const ppi_rparams &rp = d.rp[P.r];
	P.local = ent.x - rp.cell_base;
	r1 = rng(rp, round, P.r, TAG_MOVE, (uint32_t) P.local, 0u);
	r2 = rng(rp, round, P.r, TAG_MOVE, (uint32_t) P.local, 1u);
	P.i = ent.y + (int) __umulhi(r1.x, (uint32_t) ent.z);
}

/* the proposal from the draws and the mover's FP32 record (po = spos, ob oc od = sori) */
__device__ __forceinline__ void propose_from(const ppi_dev &d, Proposal &P, const U4 r1, const U4 r2, const float4 po, const float4 ob, const float4 oc,
		const float4 od) {
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	P.po = po;
	const float dm = rp.disp_max_f;
	P.disp = make_float3((u01(r1.y) - 0.5f) * dm, (u01(r1.z) - 0.5f) * dm, (u01(r1.w) - 0.5f) * dm);
	const float nx = P.po.x + P.disp.x, ny = P.po.y + P.disp.y, nz = P.po.z + P.disp.z;
	/* a move that leaves the cell is rejected: cells stay valid and same-colour cells stay independent */
	P.inside = nx >= 0.f && nx < g.wf[0] && ny >= 0.f && ny < g.wf[1] && nz >= 0.f && nz < g.wf[2];
	P.pslot = 0;
	P.q = make_float4(1.f, 0.f, 0.f, 0.f);
	if(P.inside) {
		P.pslot = __float_as_int(od.w);
		/* rotation: angle uniform in [0, Theta_max), axis uniform on the sphere (inversion method) */
		const float theta = u01(r2.x) * rp.theta_max_f;
		const float zc = 1.f - 2.f * u01(r2.y);
		const float phi = 6.283185307179586f * u01(r2.z);
		const float sr = sqrtf(fmaxf(0.f, 1.f - zc * zc));
		float sp, cph, sh, ch;
		__sincosf(phi, &sp, &cph);
		__sincosf(0.5f * theta, &sh, &ch);
		P.q = make_float4(ch, sh * sr * cph, sh * sr * sp, sh * zc);
		P.cpo[0] = ob.x;
		P.cpo[1] = ob.y;
		P.cpo[2] = ob.z;
		P.cpo[3] = ob.w;
		P.cpo[4] = oc.x;
		P.cpo[5] = oc.y;
		P.cpo[6] = oc.z;
		P.cpo[7] = oc.w;
		P.cpo[8] = od.x;
	}
}

__device__ __forceinline__ void propose(const ppi_dev &d, const int4 ent, long long round, Proposal &P) {
	const int gc = ent.x, c0 = ent.y, cnt = ent.z;
	P.r = ent.w;
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	P.local = gc - rp.cell_base;
	/* the attempt's Philox draws: particle + displacement, rotation (acceptance only when needed) */
	const U4 r1 = rng(rp, round, P.r, TAG_MOVE, (uint32_t) P.local, 0u), r2 = rng(rp, round, P.r, TAG_MOVE, (uint32_t) P.local, 1u);
	P.i = c0 + (int) __umulhi(r1.x, (uint32_t) cnt);
	P.po = ld_keep(d.spos + P.i);
	const float dm = rp.disp_max_f;
	P.disp = make_float3((u01(r1.y) - 0.5f) * dm, (u01(r1.z) - 0.5f) * dm, (u01(r1.w) - 0.5f) * dm);
	const float nx = P.po.x + P.disp.x, ny = P.po.y + P.disp.y, nz = P.po.z + P.disp.z;
	/* a move that leaves the cell is rejected: cells stay valid and same-colour cells stay independent */
	P.inside = nx >= 0.f && nx < g.wf[0] && ny >= 0.f && ny < g.wf[1] && nz >= 0.f && nz < g.wf[2];
	P.pslot = 0;
	P.q = make_float4(1.f, 0.f, 0.f, 0.f);
	if(P.inside) {
		const float4 ob = ld_keep(d.sori + 3 * (size_t) P.i), oc = ld_keep(d.sori + 3 * (size_t) P.i + 1), od = ld_keep(d.sori + 3 * (size_t) P.i + 2);
		P.pslot = __float_as_int(od.w);
		/* rotation: angle uniform in [0, Theta_max), axis uniform on the sphere (inversion method) */
		const float theta = u01(r2.x) * rp.theta_max_f;
		const float zc = 1.f - 2.f * u01(r2.y);
		const float phi = 6.283185307179586f * u01(r2.z);
		const float sr = sqrtf(fmaxf(0.f, 1.f - zc * zc));
		float sp, cph, sh, ch;
		__sincosf(phi, &sp, &cph);
		__sincosf(0.5f * theta, &sh, &ch);
		P.q = make_float4(ch, sh * sr * cph, sh * sr * sp, sh * zc);
		P.cpo[0] = ob.x;
		P.cpo[1] = ob.y;
		P.cpo[2] = ob.z;
		P.cpo[3] = ob.w;
		P.cpo[4] = oc.x;
		P.cpo[5] = oc.y;
		P.cpo[6] = oc.z;
		P.cpo[7] = oc.w;
		P.cpo[8] = od.x;
	}
}

/* FP32 rotation matrix of a unit quaternion (w, x, y, z), rows */
__device__ __forceinline__ void quatmat32(float4 q, float *Q) {
	const float w = q.x, x = q.y, y = q.z, z = q.w;
	Q[0] = 1.f - 2.f * (y * y + z * z);
	Q[1] = 2.f * (x * y - w * z);
	Q[2] = 2.f * (x * z + w * y);
	Q[3] = 2.f * (x * y + w * z);
	Q[4] = 1.f - 2.f * (x * x + z * z);
	Q[5] = 2.f * (y * z - w * x);
	Q[6] = 2.f * (x * z - w * y);
	Q[7] = 2.f * (y * z + w * x);
	Q[8] = 1.f - 2.f * (x * x + y * y);
}

/* candidate orientation columns cpn = R . Q of the old columns cpo */
__device__ __forceinline__ void cols_new(const float *cpo, float4 q, float *cpn) {
	float Q[9];
	quatmat32(q, Q);
#pragma unroll
	for(int jj = 0; jj < 3; jj++)
#pragma unroll
		for(int k3 = 0; k3 < 3; k3++) cpn[3 * jj + k3] = fmaf(cpo[k3], Q[jj], fmaf(cpo[3 + k3], Q[3 + jj], cpo[6 + k3] * Q[6 + jj]));
}

/* accepted move: FP64 q' = q (x) dq and r' = r + disp (state64 defines the same bits), FP32 record */
__device__ __forceinline__ void commit_move(const ppi_dev &d, int i, int pslot, float4 po, float3 disp, float4 q, const float *cpn) {
	double *rec = d.rec + (size_t) pslot * PPI_REC;
	const double2 r01 = *(const double2 *) rec, r23 = *(const double2 *) (rec + 2), r45 = *(const double2 *) (rec + 4);
	const double r6 = rec[6];
	const double qv[4] = { r23.y, r45.x, r45.y, r6 };
	const double b[4] = { f2d(q.x), f2d(q.y), f2d(q.z), f2d(q.w) };
	double qn[4];
#pragma unroll
	for(int c = 0; c < 4; c++) qn[c] = qcomp64(qv[c], qv[c ^ 1], qv[c ^ 2], qv[c ^ 3], b, c);
	*(double2 *) rec = make_double2(__dadd_rn(r01.x, f2d(disp.x)), __dadd_rn(r01.y, f2d(disp.y)));
	*(double2 *) (rec + 2) = make_double2(__dadd_rn(r23.x, f2d(disp.z)), qn[0]);
	*(double2 *) (rec + 4) = make_double2(qn[1], qn[2]);
	rec[6] = qn[3];
	d.spos[i] = make_float4(po.x + disp.x, po.y + disp.y, po.z + disp.z, po.w);
	d.sori[3 * (size_t) i] = make_float4(cpn[0], cpn[1], cpn[2], cpn[3]);
	d.sori[3 * (size_t) i + 1] = make_float4(cpn[4], cpn[5], cpn[6], cpn[7]);
	((float *) (d.sori + 3 * (size_t) i + 2))[0] = cpn[8];
}

/* commit_move with the mover's FP64 record already in registers (rec = its 16 doubles) */
__device__ __forceinline__ void commit_from(const ppi_dev &d, const double *rec, int i, int pslot, float4 po, float3 disp, float4 q, const float *cpn) {
	double *out = d.rec + (size_t) pslot * PPI_REC;
	const double qv[4] = { rec[PPI_Q], rec[PPI_Q + 1], rec[PPI_Q + 2], rec[PPI_Q + 3] };
	const double b[4] = { f2d(q.x), f2d(q.y), f2d(q.z), f2d(q.w) };
	double qn[4];
#pragma unroll
	for(int c = 0; c < 4; c++) qn[c] = qcomp64(qv[c], qv[c ^ 1], qv[c ^ 2], qv[c ^ 3], b, c);
	*(double2 *) out = make_double2(__dadd_rn(rec[0], f2d(disp.x)), __dadd_rn(rec[1], f2d(disp.y)));
	*(double2 *) (out + 2) = make_double2(__dadd_rn(rec[2], f2d(disp.z)), qn[0]);
	*(double2 *) (out + 4) = make_double2(qn[1], qn[2]);
	out[6] = qn[3];
	d.spos[i] = make_float4(po.x + disp.x, po.y + disp.y, po.z + disp.z, po.w);
	d.sori[3 * (size_t) i] = make_float4(cpn[0], cpn[1], cpn[2], cpn[3]);
	d.sori[3 * (size_t) i + 1] = make_float4(cpn[4], cpn[5], cpn[6], cpn[7]);
	((float *) (d.sori + 3 * (size_t) i + 2))[0] = cpn[8];
}

/* Metropolis on dE = -(bn - bo) (MC.c:332-339) */
__device__ __forceinline__ bool metropolis(const ppi_rparams &rp, long long round, int r, int local, int bo, int bn) {
	const int dE = bo - bn; /* E = -bonds */
	if(dE <= 0) return true;
	const U4 u3 = rng(rp, round, r, TAG_MOVE, (uint32_t) local, 2u);
	const uint64_t U = ((uint64_t) u3.x << 21) | (u3.y >> 11);
	return U < rp.acc_thr[dE < 31 ? dE : 31];
}

/* one whole attempt on its own, every guard-band pair decided exactly on the spot (the deferred
 * attempts; the proposal is drawn again from the same counters, so it is the same proposal) */
template <int MODE>
__device__ __forceinline__ void attempt_exact(const ppi_dev &d, const int4 ent, long long round, Acc &A) {
	Proposal P;
	propose(d, ent, round, P);
	if(!P.inside) return;
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	ppi_rstate *rs = d.rs + P.r;
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int cx = P.local % nx, cy = (P.local / nx) % ny, cz = P.local / (nx * ny);
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float rc2e = rp.sqr_rcut_f + eps, ovl = 1.f - eps;
	float cpn[9];
	cols_new(P.cpo, P.q, cpn);
	const float4 pn = make_float4(P.po.x + P.disp.x, P.po.y + P.disp.y, P.po.z + P.disp.z, 0.f);
	int bo = 0, bn = 0;
	for(int t = 0; t < 27; t++) {
		const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
		const int cell = rp.cell_base + (wrapi(cz + dz, nz) * ny + wrapi(cy + dy, ny)) * nx + wrapi(cx + dx, nx);
		const float ox = dx * g.wf[0], oy = dy * g.wf[1], oz = dz * g.wf[2];
		for(int jq = d.cell_start[cell]; jq < d.cell_start[cell + 1]; jq++) {
			if(jq == P.i) continue;
			const float4 qa = d.spos[jq];
			const float dxo = (qa.x - P.po.x) + ox, dyo = (qa.y - P.po.y) + oy, dzo = (qa.z - P.po.z) + oz;
			const float dxn = (qa.x - pn.x) + ox, dyn = (qa.y - pn.y) + oy, dzn = (qa.z - pn.z) + oz;
			const float r2o = fmaf(dxo, dxo, fmaf(dyo, dyo, dzo * dzo)), r2n = fmaf(dxn, dxn, fmaf(dyn, dyn, dzn * dzn));
			A.pairs += 2;
			if(MODE != MODE_AUDIT && r2n < ovl) return;
			if(!(MODE == MODE_AUDIT || r2o < rc2e || r2n < rc2e)) continue;
			const float4 qb = d.sori[3 * (size_t) jq], qc = d.sori[3 * (size_t) jq + 1], qd = d.sori[3 * (size_t) jq + 2];
			const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
			const int qslot = __float_as_int(qd.w);
			const int clo = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 0, P.q, P.disp, qslot, dxo, dyo, dzo, P.cpo, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr, nullptr,
					A.fallbacks);
			const int cln = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 1, P.q, P.disp, qslot, dxn, dyn, dzn, cpn, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr, nullptr,
					A.fallbacks);
			if(cln == CL_OVER) return;
			bo += (clo == CL_BOND);
			bn += (cln == CL_BOND);
		}
	}
	if(!metropolis(rp, round, P.r, P.local, bo, bn)) return;
	if(P.r != A.r) {
		flush_thread(d, A);
		A.r = P.r;
	}
	A.acc++;
	A.dbonds += bn - bo;
	commit_move(d, P.i, P.pslot, P.po, P.disp, P.q, cpn);
}

/* pair geometry: d = q - p in p's cell frame for the old (o) and candidate (n) state of attempt a */
struct PairGeo {
	float dxo, dyo, dzo, dxn, dyn, dzn;
};

template <typename SM>
__device__ __forceinline__ PairGeo pair_geo(const SM &S, int a, int t, float4 qa) {
	const float4 p = S.pos[a], m = S.md[a], w = S.wv[a];
	const int nxc = __float_as_int(w.w);
	int dxc = __float_as_int(qa.w) - __float_as_int(p.w);
	dxc = dxc > 1 ? dxc - nxc : (dxc < -1 ? dxc + nxc : dxc);
	const float ox = dxc * w.x, oy = (t % 3 - 1) * w.y, oz = (t / 3 - 1) * w.z;
	PairGeo G;
	G.dxo = (qa.x - p.x) + ox;
	G.dyo = (qa.y - p.y) + oy;
	G.dzo = (qa.z - p.z) + oz;
	G.dxn = (qa.x - (p.x + m.x)) + ox;
	G.dyn = (qa.y - (p.y + m.y)) + oy;
	G.dzn = (qa.z - (p.z + m.z)) + oz;
	return G;
}

/* old (cpo) and candidate (cpn) orientation columns of attempt a */
__device__ __forceinline__ void mover_cols(const TileSmem &S, int a, float *cpo, float *cpn) {
#pragma unroll
	for(int k = 0; k < 9; k++) cpo[k] = S.cpo[k][a];
	cols_new(cpo, S.qr[a], cpn);
}

/* patch tests of the listed close pairs, 32 per step */
template <int MODE>
__device__ __forceinline__ void tile_close(const ppi_dev &d, TileSmem &S, int lane, Acc &A) {
	const int nc = S.nc;
	for(int c = lane; c < nc; c += 32) {
		const int en = S.cbuf[c];
		const int a = (en >> 4) & 63, t = en & 15;
		if(S.flag[a] & (TF_OVER | TF_DEFER)) continue;
		const int jq = S.mi[a] + (en >> 10);
		const ppi_rparams &rp = d.rp[S.rep[a]];
		const float4 qa = ld_keep(d.spos + jq), qb = ld_keep(d.sori + 3 * (size_t) jq), qc = ld_keep(d.sori + 3 * (size_t) jq + 1), qd = ld_keep(d.sori + 3 * (size_t) jq + 2);
		const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
		const PairGeo G = pair_geo(S, a, t, qa);
		const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
		float cpo[9], cpn[9];
		mover_cols(S, a, cpo, cpn);
		int clo, cln;
		if(MODE == MODE_AUDIT) { /* test mode: every pair also through the FP64 comparison */
			ppi_rstate *rs = d.rs + S.rep[a];
			const float4 md = S.md[a];
			const int pslot = __float_as_int(md.w), qslot = __float_as_int(qd.w);
			const float3 disp = make_float3(md.x, md.y, md.z);
			clo = pair_state<MODE>(d.rec, rp, rs, d.grid[S.rep[a]].inv_L, pslot, 0, S.qr[a], disp, qslot, G.dxo, G.dyo, G.dzo, cpo, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr, nullptr, A.fallbacks);
			cln = pair_state<MODE>(d.rec, rp, rs, d.grid[S.rep[a]].inv_L, pslot, 1, S.qr[a], disp, qslot, G.dxn, G.dyn, G.dzn, cpn, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr, nullptr, A.fallbacks);
		}
		else {
			int pvo, pvn;
			clo = classify_pv(G.dxo, G.dyo, G.dzo, cpo, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, &pvo);
			cln = classify_pv(G.dxn, G.dyn, G.dzn, cpn, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, &pvn);
			/* guard band: recorded with its patch verdict, decided after the planes by the certified FP64 test */
			const int nu = (clo == CL_UNSURE) + (cln == CL_UNSURE);
			if(nu) {
				const int k = atomicAdd(&S.nu, nu);
				if(k + nu > TILE_UCAP) {
					atomicOr(&S.flag[a], TF_DEFER);
					continue;
				}
				int kk = k;
				if(clo == CL_UNSURE) S.uns[kk++] = make_int2(jq, (pvo << 7) | (a << 1));
				if(cln == CL_UNSURE) S.uns[kk] = make_int2(jq, (pvn << 7) | (a << 1) | 1);
			}
		}
		if(clo == CL_BOND) atomicAdd(&S.bo[a], 1);
		if(cln == CL_BOND) atomicAdd(&S.bn[a], 1);
		if(cln == CL_OVER) atomicOr(&S.flag[a], TF_OVER);
	}
	__syncwarp();
	if(lane == 0) S.nc = 0;
	__syncwarp();
}

/* proposal of attempt a = (list entry ent) into the tile's shared state */
__device__ __forceinline__ int tile_setup(const ppi_dev &d, TileSmem &S, int a, const int4 ent, long long round, Acc &A) {
	int flag = TF_CLOSED;
	Proposal P;
	P.i = P.r = P.local = P.pslot = 0;
	P.po = make_float4(0.f, 0.f, 0.f, 0.f);
	P.q = make_float4(1.f, 0.f, 0.f, 0.f);
	P.disp = make_float3(0.f, 0.f, 0.f);
	float4 wv = make_float4(1.f, 1.f, 1.f, __int_as_float(4));
	float2 lim = make_float2(0.f, 0.f);
	if(ent.x >= 0) {
		if(ent.w != A.r) {
			flush_thread(d, A);
			A.r = ent.w;
		}
		A.tries++;
		propose(d, ent, round, P);
		const ppi_grid &g = d.grid[P.r];
		const ppi_rparams &rp = d.rp[P.r];
		const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
		lim = make_float2(1.f - eps, rp.sqr_rcut_f + eps);
		wv = make_float4(g.wf[0], g.wf[1], g.wf[2], __int_as_float(g.n[0]));
		const int cx = P.local % g.n[0], cy = (P.local / g.n[0]) % g.n[1], cz = P.local / (g.n[0] * g.n[1]);
		S.cc[a] = cx | (cy << 10) | (cz << 20);
		if(P.inside) {
			flag = 0;
#pragma unroll
			for(int k = 0; k < 9; k++) S.cpo[k][a] = P.cpo[k];
		}
	}
	S.pos[a] = P.po;
	S.md[a] = make_float4(P.disp.x, P.disp.y, P.disp.z, __int_as_float(P.pslot));
	S.wv[a] = wv;
	S.qr[a] = P.q;
	S.mi[a] = P.i;
	S.lim[a] = lim;
	S.rep[a] = P.r;
	S.bo[a] = 0;
	S.bn[a] = 0;
	S.flag[a] = flag;
	return P.local;
}

/* the three rows (dy = -1, 0, 1) of plane dz of attempt a's neighbourhood: each row is one or two
 * contiguous ranges of sorted positions (two where the x range wraps around the box) */
struct PlaneRanges {
	int s[6], e[6];
};

__device__ __forceinline__ int plane_ranges(const ppi_dev &d, const TileSmem &S, int a, int pz, PlaneRanges &P) {
	int n = 0;
#pragma unroll
	for(int k = 0; k < 6; k++) P.s[k] = P.e[k] = 0;
	if(S.flag[a] & (TF_OVER | TF_CLOSED | TF_DEFER)) return 0;
	const int r = S.rep[a];
	const ppi_grid &g = d.grid[r];
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int cb = d.rp[r].cell_base;
	const int ccp = S.cc[a];
	const int cx = ccp & 1023, cy = (ccp >> 10) & 1023, cz = ccp >> 20;
	const bool inner = cx >= 1 && cx <= nx - 2;
	const int xa0 = inner ? cx - 1 : (cx == 0 ? nx - 1 : nx - 2), xa1 = inner ? cx + 2 : nx;
	const int xb1 = cx == 0 ? 2 : 1;
#pragma unroll
	for(int ry = 0; ry < 3; ry++) {
		const int *cs = d.cell_start + cb + (wrapi(cz + pz - 1, nz) * ny + wrapi(cy + ry - 1, ny)) * nx;
		P.s[2 * ry] = cs[xa0];
		P.e[2 * ry] = cs[xa1];
		if(!inner) {
			P.s[2 * ry + 1] = cs[0];
			P.e[2 * ry + 1] = cs[xb1];
		}
	}
#pragma unroll
	for(int k = 0; k < 6; k++) n += P.e[k] - P.s[k];
	return n;
}

/* attempt a's pairs of plane pz into the pair list from position pos */
__device__ __forceinline__ void write_pairs(TileSmem &S, int a, int pz, const PlaneRanges &P, int pos) {
	const int i = S.mi[a];
#pragma unroll
	for(int sg = 0; sg < 6; sg++) {
		const int tag = (a << 4) | (3 * pz + (sg >> 1));
		for(int jq = P.s[sg]; jq < P.e[sg]; jq++) {
			const int off = jq - i;
			if(off >= TILE_OFF_MAX || off <= -TILE_OFF_MAX) {
				atomicOr(&S.flag[a], TF_DEFER);
				S.pbuf[pos++] = tag; /* offset 0 = the mover itself: skipped */
			}
			else S.pbuf[pos++] = (int) ((unsigned) off << 10) | tag;
		}
	}
}

/* remembers deferred attempt list index e */
__device__ __forceinline__ void defer_attempt(const ppi_dev &d, TileSmem &S, int col, int e) {
	const int k = atomicAdd(&S.nd, 1);
	if(k < TILE_DCAP) S.dl[k] = e;
	else {
		d.dflag[(size_t) col * d.clist_cap + e] = 1;
		S.dov = 1;
	}
}

/* the pair list's np entries, PSTEP steps of 32 pairs at a time: distance filter, certain overlaps,
 * close pairs compacted into the patch-test list */
template <int MODE>
__device__ __forceinline__ void tile_steps(const ppi_dev &d, TileSmem &S, const int lane, const int np, Acc &A) {
	const unsigned lt = (1u << lane) - 1u;
	/* PSTEP steps of 32 pairs at a time: the candidate loads of all of them are issued before any is
	 * used, so that a step group costs one memory latency instead of PSTEP */
	for(int p0 = 0; p0 < np; p0 += 32 * PSTEP) {
		int en[PSTEP], ok[PSTEP];
		float4 qa[PSTEP];
#pragma unroll
		for(int u = 0; u < PSTEP; u++) {
			const int p = p0 + 32 * u + lane;
			en[u] = 0;
			ok[u] = 0;
			qa[u] = make_float4(0.f, 0.f, 0.f, 0.f);
			if(p < np) {
				en[u] = S.pbuf[p];
				const int a = (en[u] >> 4) & 63, off = en[u] >> 10;
				ok[u] = off != 0 && !(S.flag[a] & (TF_OVER | TF_DEFER));
				if(ok[u]) qa[u] = ld_keep(d.spos + (S.mi[a] + off));
			}
		}
		int close[PSTEP];
#pragma unroll
		for(int u = 0; u < PSTEP; u++) {
			close[u] = 0;
			if(ok[u]) {
				const int a = (en[u] >> 4) & 63;
				const PairGeo G = pair_geo(S, a, en[u] & 15, qa[u]);
				const float r2o = fmaf(G.dxo, G.dxo, fmaf(G.dyo, G.dyo, G.dzo * G.dzo));
				const float r2n = fmaf(G.dxn, G.dxn, fmaf(G.dyn, G.dyn, G.dzn * G.dzn));
				const float2 lim = S.lim[a];
				A.pairs += 2;
				if(MODE != MODE_AUDIT && r2n < lim.x) atomicOr(&S.flag[a], TF_OVER); /* certain overlap of the candidate state */
				else close[u] = MODE == MODE_AUDIT || r2o < lim.y || r2n < lim.y;
			}
		}
		/* compact the group's close pairs into the patch-test list */
		unsigned m[PSTEP];
		int tot = 0;
#pragma unroll
		for(int u = 0; u < PSTEP; u++) {
			m[u] = __ballot_sync(0xffffffffu, close[u]);
			tot += __popc(m[u]);
		}
		if(tot) {
			if(S.nc + tot > TILE_CCAP) tile_close<MODE>(d, S, lane, A);
			int base = S.nc;
#pragma unroll
			for(int u = 0; u < PSTEP; u++) {
				if(close[u]) S.cbuf[base + __popc(m[u] & lt)] = en[u];
				base += __popc(m[u]);
			}
			__syncwarp();
			if(lane == 0) S.nc = base;
			__syncwarp();
		}
	}
}

/* attempt a's pairs from its mover's neighbour list (n entries) into the pair list from position pos, in
 * the packing of write_pairs: the row tag of an entry with cell offset code c is c / 3 ((dy + 1) +
 * 3 (dz + 1)); pair_geo recovers dx from the cells' x indices */
__device__ __forceinline__ void write_list_pairs(const ppi_dev &d, TileSmem &S, int a, int n, int pos) {
	const int i = S.mi[a];
	const int4 *L = (const int4 *) (d.nl + (size_t) i * d.nl_k);
	for(int k0 = 0; k0 < n; k0 += 32) { /* up to 32 entries' loads at once: one latency for a list */
		int4 v[8];
#pragma unroll
		for(int c = 0; c < 8; c++) v[c] = (k0 + 4 * c < n) ? ld_stream(L + (k0 >> 2) + c) : make_int4(0, 0, 0, 0);
#pragma unroll
		for(int c = 0; c < 8; c++) {
			const int e4[4] = { v[c].x, v[c].y, v[c].z, v[c].w };
#pragma unroll
			for(int u = 0; u < 4; u++) {
				const int k = k0 + 4 * c + u;
				if(k >= n) continue;
				const int jq = (int) ((unsigned) e4[u] >> 5), code = e4[u] & 31;
				const int off = jq - i, tag = (a << 4) | (code / 3);
				if(off >= TILE_OFF_MAX || off <= -TILE_OFF_MAX) {
					atomicOr(&S.flag[a], TF_DEFER);
					S.pbuf[pos + k] = tag; /* offset 0 = the mover itself: skipped */
				}
				else S.pbuf[pos + k] = (int) ((unsigned) off << 10) | tag;
			}
		}
	}
}

/* the TA attempts of list positions b + lane (e0) and b + 32 + lane (e1); ent.x < 0: none */
template <int MODE, bool LIST>
__device__ __forceinline__ void tile_round(const ppi_dev &d, TileSmem &S, const int lane, const int4 e0, const int4 e1, int b, int col, long long round, Acc &A,
		bool &waited) {
	const int loc0 = tile_setup(d, S, lane, e0, round, A);
	const int loc1 = tile_setup(d, S, lane + 32, e1, round, A);
	if(!waited && !LIST) { /* the proposals are drawn: from here on the previous colour's moves must be complete */
		grid_dep_wait();
		grid_dep_release();
		waited = true;
	}
	if(lane == 0) {
		S.nc = 0;
		S.nu = 0;
	}
	__syncwarp();
	if(LIST) {
		/* the pairs come from the movers' neighbour lists, one half of the attempts (a lane each) at a time */
#pragma unroll 1
		for(int h = 0; h < 2; h++) {
			const int a = lane + 32 * h;
			int n = 0;
			if(!(S.flag[a] & (TF_OVER | TF_CLOSED | TF_DEFER))) {
				n = d.nl_cnt[S.mi[a]];
				if(n > d.nl_k) { /* the list overflowed: the exact 27-cell path */
					atomicOr(&S.flag[a], TF_DEFER);
					n = 0;
				}
			}
			int incl = n;
#pragma unroll
			for(int o = 1; o < 32; o <<= 1) {
				const int v = __shfl_up_sync(0xffffffffu, incl, o);
				if(lane >= o) incl += v;
			}
			const int total = __shfl_sync(0xffffffffu, incl, 31);
			/* lanes whose slices fit the pair list together (a slice is at most nl_k <= 128 < TILE_PCAP) */
			int done = 0;
			while(done < total) {
				const int start = incl - n;
				const int mine = n > 0 && start >= done && incl - done <= TILE_PCAP;
				const unsigned take = __ballot_sync(0xffffffffu, mine);
				if(take == 0) break; /* unreachable while nl_k <= TILE_PCAP */
				if(mine) write_list_pairs(d, S, a, n, start - done);
				const int end = __shfl_sync(0xffffffffu, incl, 31 - __clz(take));
				__syncwarp();
				if(!waited) { /* the epoch's lists are read: the candidates need the previous colour complete */
					grid_dep_wait();
					grid_dep_release();
					waited = true;
				}
				tile_steps<MODE>(d, S, lane, end - done, A);
				done = end;
				__syncwarp();
			}
		}
	}
#pragma unroll 1
	for(int pz = 0; pz < (LIST ? 0 : 3); pz++) {
		PlaneRanges P0, P1;
		const int n0 = plane_ranges(d, S, lane, pz, P0);
		const int n1 = plane_ranges(d, S, lane + 32, pz, P1);
		const int n = n0 + n1;
		int incl = n;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1) {
			const int v = __shfl_up_sync(0xffffffffu, incl, o);
			if(lane >= o) incl += v;
		}
		if(__shfl_sync(0xffffffffu, incl, 31) == 0) continue;
		/* the lanes whose slices fit into the list; the others' attempts are deferred (dense corner case) */
		const unsigned fit = __ballot_sync(0xffffffffu, incl <= TILE_PCAP);
		const int np = fit ? __shfl_sync(0xffffffffu, incl, 31 - __clz(fit)) : 0;
		if(incl > TILE_PCAP) {
			if(n0) atomicOr(&S.flag[lane], TF_DEFER);
			if(n1) atomicOr(&S.flag[lane + 32], TF_DEFER);
		}
		else {
			const int pos = incl - n;
			write_pairs(S, lane, pz, P0, pos);
			write_pairs(S, lane + 32, pz, P1, pos + n0);
		}
		__syncwarp();
		tile_steps<MODE>(d, S, lane, np, A);
	}
	if(!waited) { /* no pair of this iteration read a neighbour: wait before the decisions and commits */
		grid_dep_wait();
		grid_dep_release();
		waited = true;
	}
	if(S.nc) tile_close<MODE>(d, S, lane, A);
	/* guard-band pairs: certified FP64 decisions (no division chain), the whole warp on each pair; an
	 * undecided one defers its attempt */
	if(MODE == MODE_FAST) {
		const int nu = S.nu < TILE_UCAP ? S.nu : TILE_UCAP;
#pragma unroll 1
		for(int u = 0; u < nu; u++) {
			const int2 v = S.uns[u];
			const int jq = v.x, a = (v.y >> 1) & 63, kind = v.y & 1, pv = v.y >> 7;
			if(S.flag[a] & (TF_OVER | TF_DEFER)) continue; /* warp-uniform: read after the last __syncwarp */
			const int r = S.rep[a];
			const float4 md = S.md[a];
			const int ex = decide64_warp(d.rec, d.rp[r], d.rs[r].box, d.grid[r].inv_L, __float_as_int(md.w), kind, S.qr[a], make_float3(md.x, md.y, md.z),
					__float_as_int(d.sori[3 * (size_t) jq + 2].w), 0, nullptr, nullptr, lane, pv);
			if(lane == 0) {
				A.fallbacks++;
				if(ex == DEC64_EXACT) atomicOr(&S.flag[a], TF_DEFER);
				else if(ex == 1) atomicAdd(kind ? &S.bn[a] : &S.bo[a], 1);
				else if(ex == -1 && kind) atomicOr(&S.flag[a], TF_OVER);
			}
			__syncwarp();
		}
	}
	/* decisions and commits of the attempts that are not deferred */
#pragma unroll 1
	for(int k = 0; k < 2; k++) {
		const int a = lane + 32 * k;
		const int flag = S.flag[a];
		if(flag & (TF_OVER | TF_CLOSED)) continue;
		if(flag & TF_DEFER) {
			defer_attempt(d, S, col, b + a);
			continue;
		}
		const int r = S.rep[a];
		const int bo = S.bo[a], bn = S.bn[a];
		if(!metropolis(d.rp[r], round, r, k ? loc1 : loc0, bo, bn)) continue;
		if(r != A.r) {
			flush_thread(d, A);
			A.r = r;
		}
		A.acc++;
		A.dbonds += bn - bo;
		float cpo[9], cpn[9];
		mover_cols(S, a, cpo, cpn);
		const float4 md = S.md[a];
		commit_move(d, S.mi[a], __float_as_int(md.w), S.pos[a], make_float3(md.x, md.y, md.z), S.qr[a], cpn);
	}
}

/* one colour of a round: the colour's non-empty cells, TA per warp and iteration */
template <int MODE, bool LIST>
__global__ void __launch_bounds__(32 * TILE_WARPS, MODE == MODE_FAST ? PPI_TILE_MIN_BLOCKS : 1) k_colour(ppi_dev d, long long round, int col) {
	if(round < 0) { /* graph launch: round after the device counter, col = slot in the round's colour order */
		round = ctr_index(round, d.ctr->round);
		col = colour_at(round, col);
	}
	__shared__ TileSmem s_tile[TILE_WARPS];
	TileSmem &S = s_tile[threadIdx.x >> 5];
	const int lane = threadIdx.x & 31;
	const int4 *list = d.clist + (size_t) col * d.clist_cap;
	int cnt = d.ccount[col];
	if(cnt > d.clist_cap) cnt = d.clist_cap;
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
	/* every resident warp gets an equal share of the list (the CTA scheduler does not spread the
	 * working CTAs of a partly filled grid evenly over the SMs) */
	const int lo = (int) ((long long) warp * cnt / nwarp), hi = (int) ((long long) (warp + 1) * cnt / nwarp);
	const int4 none = make_int4(-1, 0, 0, 0);
	if(lane == 0) {
		S.nd = 0;
		S.dov = 0;
	}
	__syncwarp();
	bool waited = false;
	for(int b = lo; b < hi; b += TA) {
		const int4 e0 = (b + lane < hi) ? ld_stream(list + b + lane) : none;
		const int4 e1 = (b + 32 + lane < hi) ? ld_stream(list + b + 32 + lane) : none;
		tile_round<MODE, LIST>(d, S, lane, e0, e1, b, col, round, A, waited);
		__syncwarp();
	}
	if(!waited) {
		grid_dep_wait();
		grid_dep_release();
	}
	/* the deferred attempts, one per lane, exactly */
	const int nd = S.nd < TILE_DCAP ? S.nd : TILE_DCAP;
	for(int k = lane; k < nd; k += 32) attempt_exact<MODE>(d, list[S.dl[k]], round, A);
	if(S.dov) {
		unsigned char *fl = d.dflag + (size_t) col * d.clist_cap;
		for(int e = lo + lane; e < hi; e += 32)
			if(fl[e]) {
				fl[e] = 0;
				attempt_exact<MODE>(d, list[e], round, A);
			}
	}
	__syncwarp();
	flush_block(d, A);
}

/* ------------------------------------------------------------------------------------------------ */
/* persistent round over the neighbour lists (k_round)                                              */
/* ------------------------------------------------------------------------------------------------ */
/* The 8 colours of a plain round in one cooperative launch, with a grid barrier between colours. A warp
 * takes 32 attempts at a time (one per lane) and moves each step's global reads into shared memory with
 * cp.async before it computes on them, so that a step costs one memory latency however many pairs it has:
 *   1. proposal: the movers' FP32 records, list lengths and first KR_NL0 list entries, all loaded
 *      together (registers); the movers' FP64 records start towards shared memory;
 *   2. the candidate positions of every listed pair -> shared memory; distance filter, certain overlaps,
 *      close pairs compacted;
 *   3. the close candidates' orientation records -> shared memory; patch tests; guard-band pairs go to the
 *      certified FP64 test; decisions; commits from the staged FP64 records.
 * Step 1 of a colour's first iteration runs before the barrier that closes the previous colour: it reads
 * only its own movers (the previous colour moves none of them) and the epoch's lists. The per-pair
 * decisions are k_colour's (the same classify, guard band, decide64 and exact_pair on the same proposals)
 * and every decision is the exact one, so the trajectory equals k_colour's bit for bit; an attempt
 * k_colour would defer (list overflow, guard-band pairs beyond KR_UCAP) takes the same exact path.
 * Barrier: a CTA arrives once per colour (after __syncthreads, a gpu-scope fence and an atomic add); a
 * CTA waits by one thread spinning with acquire loads, then __syncthreads. Every wait is bounded by
 * d.bar_limit SM cycles: one that runs out writes PPI_E_BARRIER to gbar[15] and its CTA returns (the others
 * then run out at their next wait), so a missing CTA can never hang the GPU. The launch is cooperative,
 * so every CTA of the grid is resident. */
#define KR_WARPS 4
#define KR_A 32      /* attempts per warp iteration: one per lane */
#define KR_PCAP 512  /* staged candidate positions per chunk of an iteration's pairs */
#define KR_CCAP 128  /* staged close-pair orientation records per chunk */
#define KR_NL0 32    /* list entries loaded with the proposal, all in one step (the rest, if any, in the pair step) */
#define KR_UCAP 32   /* guard-band pairs per iteration decided in place (more: the attempt is deferred) */
#define KR_DCAP 64   /* deferred attempts a warp keeps (flushed once more than KR_DCAP - KR_A are waiting) */
#define KR_LIMIT_DEFAULT (1ll << 31) /* SM clock cycles of a barrier wait: ~1 s at 2 GHz */

struct __align__(16) RoundSmem {
	float4 qpos[KR_PCAP];       /* staged candidate positions (spos) */
	float4 qori[3 * KR_CCAP];   /* staged close candidates' orientation records (sori) */
	double mrec[KR_A][8];       /* staged movers' FP64 records, doubles 0..7 (x y z q) */
	float4 pos[KR_A];           /* old cell-local position, .w = cell x index */
	float4 md[KR_A];            /* displacement, .w = mover slot */
	float4 wv[KR_A];            /* cell edges, .w = number of x cells */
	float4 qr[KR_A];            /* proposed rotation quaternion */
	float cpo[9][KR_A];         /* mover's old orientation columns */
	float cpn[9][KR_A];         /* mover's candidate orientation columns */
	float2 lim[KR_A];           /* (1 - eps, r_cut^2 + eps) */
	int pj[KR_PCAP];            /* candidate sorted position of pair p */
	unsigned short pat[KR_PCAP]; /* attempt << 4 | row (dy + 1) + 3 (dz + 1) of pair p */
	short cl[KR_PCAP];          /* the close pairs (indices p) */
	int mi[KR_A], rep[KR_A], flag[KR_A], bo[KR_A], bn[KR_A];
	int2 uns[KR_UCAP];          /* guard-band pairs: (candidate sorted position, attempt << 1 | kind) */
	int dl[KR_DCAP];            /* list indices of deferred attempts */
	int nu, nd, pad, total;     /* total: listed pairs of the iteration */
};

/* 16 bytes global -> shared, through L2 only (cp.async.cg); completed by kr_cp_wait */
__device__ __forceinline__ void kr_cp16(void *dst, const void *src) {
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned) __cvta_generic_to_shared(dst)), "l"(src) : "memory");
}

/* waits for every cp.async this thread issued; the caller then __syncwarp()s before other lanes read */
__device__ __forceinline__ void kr_cp_wait() { asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory"); }

/* list entry (candidate << 5 | cell offset code) of attempt a at pair slot p */
__device__ __forceinline__ void kr_put(RoundSmem &S, int p, int entry, int a) {
	const unsigned u = (unsigned) entry;
	S.pj[p] = (int) (u >> 5);
	S.pat[p] = (unsigned short) ((a << 4) | ((u & 31u) / 3u));
}

/* step 1 for the lane's attempt (list entry ent; ent.x < 0: none): the proposal into shared memory, the
 * mover's FP64 record started towards S.mrec, and the attempt's first KR_NL0 list entries written to the
 * pair list at the attempt's slice (those that fall into the first chunk). Returns the attempt's number of
 * listed pairs n (0 if it has none or takes the exact path) and its slice's start; S.total = all pairs. */
__device__ __forceinline__ int kr_setup(const ppi_dev &d, RoundSmem &S, const int a, const int4 ent, long long round, Acc &A, int &start, int &loc) {
	int flag = TF_CLOSED, n = 0;
	int e[KR_NL0];
	Proposal P;
	P.i = P.r = P.local = P.pslot = 0;
	P.po = make_float4(0.f, 0.f, 0.f, 0.f);
	P.q = make_float4(1.f, 0.f, 0.f, 0.f);
	P.disp = make_float3(0.f, 0.f, 0.f);
	float4 wv = make_float4(1.f, 1.f, 1.f, __int_as_float(4));
	float2 lim = make_float2(0.f, 0.f);
#pragma unroll
	for(int k = 0; k < KR_NL0; k++) e[k] = 0;
	if(ent.x >= 0) {
		if(ent.w != A.r) {
			flush_thread(d, A);
			A.r = ent.w;
		}
		A.tries++;
		U4 r1, r2;
		propose_draws(d, ent, round, P, r1, r2);
		const size_t i = (size_t) P.i;
		const int K = d.nl_k;
		/* every load of the step at once: they all depend on the mover only */
		const float4 po = __ldcg(d.spos + i);
		const float4 ob = __ldcg(d.sori + 3 * i), oc = __ldcg(d.sori + 3 * i + 1), od = __ldcg(d.sori + 3 * i + 2);
		const int cnt = __ldcg(d.nl_cnt + i);
		const int4 *L = (const int4 *) (d.nl + i * (size_t) K);
		int4 v[KR_NL0 / 4];
#pragma unroll
		for(int c = 0; c < KR_NL0 / 4; c++) v[c] = (4 * c < K) ? __ldcg(L + c) : make_int4(0, 0, 0, 0);
		propose_from(d, P, r1, r2, po, ob, oc, od);
		const ppi_grid &g = d.grid[P.r];
		const ppi_rparams &rp = d.rp[P.r];
		const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
		lim = make_float2(1.f - eps, rp.sqr_rcut_f + eps);
		wv = make_float4(g.wf[0], g.wf[1], g.wf[2], __int_as_float(g.n[0]));
		if(P.inside) {
			float cpn[9];
			cols_new(P.cpo, P.q, cpn);
#pragma unroll
			for(int k = 0; k < 9; k++) {
				S.cpo[k][a] = P.cpo[k];
				S.cpn[k][a] = cpn[k];
			}
			if(cnt > K) flag = TF_DEFER; /* the list overflowed: the exact 27-cell path */
			else {
				flag = 0;
				n = cnt;
			}
			const double *rec = d.rec + (size_t) P.pslot * PPI_REC;
#pragma unroll
			for(int c = 0; c < 4; c++) kr_cp16(&S.mrec[a][2 * c], rec + 2 * c);
		}
#pragma unroll
		for(int c = 0; c < KR_NL0 / 4; c++) {
			e[4 * c] = v[c].x;
			e[4 * c + 1] = v[c].y;
			e[4 * c + 2] = v[c].z;
			e[4 * c + 3] = v[c].w;
		}
	}
	S.pos[a] = P.po;
	S.md[a] = make_float4(P.disp.x, P.disp.y, P.disp.z, __int_as_float(P.pslot));
	S.wv[a] = wv;
	S.qr[a] = P.q;
	S.mi[a] = P.i;
	S.lim[a] = lim;
	S.rep[a] = P.r;
	S.bo[a] = 0;
	S.bn[a] = 0;
	S.flag[a] = flag;
	loc = P.local;
	/* the attempts' slices of the pair list: a warp scan of the list lengths */
	int incl = n;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		const int v = __shfl_up_sync(0xffffffffu, incl, o);
		if(a >= o) incl += v;
	}
	start = incl - n;
	if(a == 31) S.total = incl;
#pragma unroll
	for(int k = 0; k < KR_NL0; k++)
		if(k < n && start + k < KR_PCAP) kr_put(S, start + k, e[k], a);
	return n;
}

/* patch tests of staged close pair q (pair p) */
__device__ __forceinline__ void kr_close(const ppi_dev &d, RoundSmem &S, int q, int p, Acc &A) {
	const int at = S.pat[p], a = at >> 4;
	if(S.flag[a] & (TF_OVER | TF_DEFER)) return;
	const float4 qb = S.qori[3 * q], qc = S.qori[3 * q + 1], qd = S.qori[3 * q + 2];
	const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
	const PairGeo G = pair_geo(S, a, at & 15, S.qpos[p]);
	const ppi_rparams &rp = d.rp[S.rep[a]];
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	float cpo[9], cpn[9];
#pragma unroll
	for(int k = 0; k < 9; k++) {
		cpo[k] = S.cpo[k][a];
		cpn[k] = S.cpn[k][a];
	}
	const int clo = classify(G.dxo, G.dyo, G.dzo, cpo, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, nullptr);
	const int cln = classify(G.dxn, G.dyn, G.dzn, cpn, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, nullptr);
	const int nu = (clo == CL_UNSURE) + (cln == CL_UNSURE);
	if(nu) { /* guard band: decided after the pairs by the certified FP64 test */
		const int k = atomicAdd(&S.nu, nu);
		if(k + nu > KR_UCAP) {
			atomicOr(&S.flag[a], TF_DEFER);
			return;
		}
		int kk = k;
		if(clo == CL_UNSURE) S.uns[kk++] = make_int2(S.pj[p], a << 1);
		if(cln == CL_UNSURE) S.uns[kk] = make_int2(S.pj[p], (a << 1) | 1);
	}
	if(clo == CL_BOND) atomicAdd(&S.bo[a], 1);
	if(cln == CL_BOND) atomicAdd(&S.bn[a], 1);
	if(cln == CL_OVER) atomicOr(&S.flag[a], TF_OVER);
}

/* remembers deferred attempt list index e (the warp flushes its list before it can overflow) */
__device__ __forceinline__ void kr_defer(RoundSmem &S, int e) { S.dl[atomicAdd(&S.nd, 1)] = e; }

/* the warp's deferred attempts, one per lane, each exactly on its own (same-colour attempts are
 * independent, so when they run does not matter) */
__device__ __forceinline__ void kr_flush_deferred(const ppi_dev &d, RoundSmem &S, const int4 *list, const int lane, long long round, Acc &A) {
	__syncwarp();
	const int nd = S.nd;
	for(int k = lane; k < nd; k += 32) attempt_exact<MODE_FAST>(d, list[S.dl[k]], round, A);
	__syncwarp();
	if(lane == 0) S.nd = 0;
	__syncwarp();
}

/* steps 2 and 3 of the iteration whose step 1 left n pairs and list entries e[] in this lane */
__device__ __forceinline__ void kr_iteration(const ppi_dev &d, RoundSmem &S, const int lane, const int n, const int start, const int loc, const int b,
		long long round, Acc &A) {
	const unsigned lt = (1u << lane) - 1u;
	__syncwarp();
	const int total = S.total;
	if(lane == 0) S.nu = 0;
	const int *Lg = d.nl + (size_t) S.mi[lane] * d.nl_k;
	for(int c0 = 0; c0 < total; c0 += KR_PCAP) {
		const int np = min(total - c0, KR_PCAP);
		/* this lane's list entries that fall into the chunk and are not written yet (kr_setup wrote the
		 * first KR_NL0 of each attempt that fall into the first chunk) */
		const int k0 = max(0, c0 - start), k1 = min(n, c0 + np - start);
		for(int k = (c0 == 0 ? max(k0, KR_NL0) : k0); k < k1; k++) kr_put(S, start + k - c0, __ldcg(Lg + k), lane);
		__syncwarp();
		/* step 2: candidate positions (and, in the first chunk, the movers' FP64 records) */
		for(int p = lane; p < np; p += 32) kr_cp16(&S.qpos[p], d.spos + S.pj[p]);
		kr_cp_wait();
		__syncwarp();
		int ncl = 0;
		for(int p0 = 0; p0 < np; p0 += 32) {
			const int p = p0 + lane;
			int close = 0;
			if(p < np) {
				const int at = S.pat[p], a = at >> 4;
				if(!(S.flag[a] & (TF_OVER | TF_DEFER))) {
					const PairGeo G = pair_geo(S, a, at & 15, S.qpos[p]);
					const float r2o = fmaf(G.dxo, G.dxo, fmaf(G.dyo, G.dyo, G.dzo * G.dzo));
					const float r2n = fmaf(G.dxn, G.dxn, fmaf(G.dyn, G.dyn, G.dzn * G.dzn));
					const float2 lim = S.lim[a];
					A.pairs += 2;
					if(r2n < lim.x) atomicOr(&S.flag[a], TF_OVER); /* certain overlap of the candidate state */
					else close = r2o < lim.y || r2n < lim.y;
				}
			}
			const unsigned m = __ballot_sync(0xffffffffu, close);
			if(close) S.cl[ncl + __popc(m & lt)] = (short) p;
			ncl += __popc(m);
		}
		__syncwarp();
		/* step 3: the close pairs' orientation records, then their patch tests */
		for(int q0 = 0; q0 < ncl; q0 += KR_CCAP) {
			const int nq = min(ncl - q0, KR_CCAP);
			for(int q = lane; q < nq; q += 32) {
				const int p = S.cl[q0 + q];
				if(S.flag[S.pat[p] >> 4] & (TF_OVER | TF_DEFER)) continue;
				const float4 *src = d.sori + 3 * (size_t) S.pj[p];
				kr_cp16(S.qori + 3 * q, src);
				kr_cp16(S.qori + 3 * q + 1, src + 1);
				kr_cp16(S.qori + 3 * q + 2, src + 2);
			}
			kr_cp_wait();
			__syncwarp();
			for(int q = lane; q < nq; q += 32) kr_close(d, S, q, S.cl[q0 + q], A);
			__syncwarp();
		}
	}
	if(total == 0) { /* no pair: the movers' FP64 records still have to arrive */
		kr_cp_wait();
		__syncwarp();
	}
	/* guard-band pairs: certified FP64 decisions, the whole warp on each pair; an undecided one defers its
	 * attempt */
	const int nu = S.nu < KR_UCAP ? S.nu : KR_UCAP;
#pragma unroll 1
	for(int u = 0; u < nu; u++) {
		const int2 v = S.uns[u];
		const int jq = v.x, a = v.y >> 1, kind = v.y & 1;
		if(S.flag[a] & (TF_OVER | TF_DEFER)) continue; /* warp-uniform: read after the last __syncwarp */
		const int r = S.rep[a];
		const float4 md = S.md[a];
		const int ex = decide64_warp(d.rec, d.rp[r], d.rs[r].box, d.grid[r].inv_L, __float_as_int(md.w), kind, S.qr[a], make_float3(md.x, md.y, md.z),
				__float_as_int(__ldcg(d.sori + 3 * (size_t) jq + 2).w), 0, nullptr, nullptr, lane);
		if(lane == 0) {
			A.fallbacks++;
			if(ex == DEC64_EXACT) atomicOr(&S.flag[a], TF_DEFER);
			else if(ex == 1) atomicAdd(kind ? &S.bn[a] : &S.bo[a], 1);
			else if(ex == -1 && kind) atomicOr(&S.flag[a], TF_OVER);
		}
		__syncwarp();
	}
	__syncwarp();
	/* decision and commit of the lane's attempt */
	const int a = lane, flag = S.flag[a];
	if(flag & (TF_OVER | TF_CLOSED)) return;
	if(flag & TF_DEFER) {
		kr_defer(S, b + a);
		return;
	}
	const int r = S.rep[a];
	const int bo = S.bo[a], bn = S.bn[a];
	if(!metropolis(d.rp[r], round, r, loc, bo, bn)) return;
	if(r != A.r) {
		flush_thread(d, A);
		A.r = r;
	}
	A.acc++;
	A.dbonds += bn - bo;
	float cpn[9];
#pragma unroll
	for(int k = 0; k < 9; k++) cpn[k] = S.cpn[k][a];
	const float4 md = S.md[a];
	commit_from(d, S.mrec[a], S.mi[a], __float_as_int(md.w), S.pos[a], make_float3(md.x, md.y, md.z), S.qr[a], cpn);
}

/* waits until gbar[0] >= target (every CTA has closed the previous colour); false if the wait ran out */
__device__ __forceinline__ bool kr_barrier_wait(const ppi_dev &d, unsigned target, long long limit, int *s_abort) {
	if(threadIdx.x == 0) {
		const long long t0 = clock64();
		unsigned ns = 32;
		for(;;) {
			unsigned v;
			asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(d.gbar) : "memory");
			if(v >= target) break;
			if(clock64() - t0 > limit) {
				atomicExch(d.gbar + 15, PPI_E_BARRIER);
				*s_abort = 1;
				break;
			}
			__nanosleep(ns);
			if(ns < 512) ns <<= 1;
		}
	}
	__syncthreads();
	return *s_abort == 0;
}

/* one plain round over the epoch's neighbour lists; colours = the round's colour order, 3 bits per slot
 * (stream launches), or round < 0 for a captured graph launch (round after the device counter, colour
 * order computed here) */
__global__ void __launch_bounds__(32 * KR_WARPS, 2) k_round(ppi_dev d, long long round, int colours) {
	const bool graph = round < 0;
	if(graph) round = ctr_index(round, d.ctr->round);
	extern __shared__ __align__(16) unsigned char kr_smem[];
	RoundSmem &S = ((RoundSmem *) kr_smem)[threadIdx.x >> 5];
	__shared__ int s_abort;
	const int lane = threadIdx.x & 31;
	const long long limit = d.bar_limit > 0 ? d.bar_limit : KR_LIMIT_DEFAULT;
	const int4 none = make_int4(-1, 0, 0, 0);
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	if(threadIdx.x == 0) s_abort = 0;
	for(int ci = 0; ci < 8; ci++) {
		const int col = graph ? colour_at(round, ci) : (colours >> (3 * ci)) & 7;
		const int4 *list = d.clist + (size_t) col * d.clist_cap;
		int cnt = d.ccount[col];
		if(cnt > d.clist_cap) cnt = d.clist_cap;
		/* iterations of KR_A list entries, handed out one at a time from the colour's work counter
		 * (gbar[1 + ci]); a warp fetches its next one while it works on the current one */
		const int nit = (cnt + KR_A - 1) / KR_A;
		unsigned *work = (unsigned *) d.gbar + 1 + ci;
		if(lane == 0) S.nd = 0;
		/* lane 0 keeps the counter's answer in a register and the warp reads it one iteration later, so
		 * the atomic's latency hides behind the work */
		unsigned pend = 0;
		if(lane == 0) pend = atomicAdd(work, 1u);
		int it = (int) __shfl_sync(0xffffffffu, pend, 0);
		if(lane == 0 && it < nit) pend = atomicAdd(work, 1u);
		int loc = 0, start = 0, n = 0;
		if(it < nit) n = kr_setup(d, S, lane, it * KR_A + lane < cnt ? list[it * KR_A + lane] : none, round, A, start, loc);
		if(ci > 0 && !kr_barrier_wait(d, (unsigned) (ci * gridDim.x + (ci == 1 ? d.bar_extra : 0)), limit, &s_abort)) return;
		while(it < nit) {
			const int nxt = (int) __shfl_sync(0xffffffffu, pend, 0);
			const int4 next = nxt < nit && nxt * KR_A + lane < cnt ? list[nxt * KR_A + lane] : none;
			if(lane == 0 && nxt < nit) pend = atomicAdd(work, 1u);
			kr_iteration(d, S, lane, n, start, loc, it * KR_A, round, A);
			__syncwarp();
			if(S.nd > KR_DCAP - KR_A) kr_flush_deferred(d, S, list, lane, round, A);
			it = nxt;
			if(it < nit) n = kr_setup(d, S, lane, next, round, A, start, loc);
		}
		kr_flush_deferred(d, S, list, lane, round, A);
		/* close the colour: every warp of the CTA is done, its writes are visible at gpu scope */
		__syncthreads();
		if(threadIdx.x == 0) {
			__threadfence();
			atomicAdd((unsigned *) d.gbar, 1u);
		}
	}
	__syncwarp();
	flush_block(d, A);
}

/* ------------------------------------------------------------------------------------------------ */
/* per-epoch neighbour lists                                                                        */
/* ------------------------------------------------------------------------------------------------ */
/* Within an epoch (the rounds between two re-sorts) no particle leaves its cell and each moves at most
 * once per round, by at most sqrt(3)/2 Disp_max (plus the NPT rescalings of accepted volume moves). The
 * host sizes the list radius (rp.nl_r2f, ppgpu_host.c: nl_radius2) so that a pair farther apart when the
 * list is built can neither overlap nor bond at any time of the epoch and stays outside the FP32 guard
 * band. k_colour<MODE, true> then takes its pairs from the movers' lists instead of the 27 cells: the
 * same decisions, hence the same trajectory, with fewer pair tests and no cell-range lookups. */
#define NL_B 128 /* threads per CTA of the list build */

/* the candidates of sorted position i in its 27 cells: visit(jq, code) for each, code = (dx + 1) +
 * 3 (dy + 1) + 9 (dz + 1). The 3 cells of a row are one contiguous range of sorted positions (two where the
 * row wraps around the box); a candidate's x offset comes from its cell's x index (spos.w). */
template <typename V>
__device__ __forceinline__ void nl_rows(const ppi_dev &d, int i, const ppi_rparams &rp, const ppi_grid &g, int cx, int cy, int cz, V visit) {
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const bool inner = cx >= 1 && cx <= nx - 2;
	const int xa0 = inner ? cx - 1 : (cx == 0 ? nx - 1 : nx - 2), xa1 = inner ? cx + 2 : nx;
	const int xb1 = cx == 0 ? 2 : 1;
#pragma unroll 1
	for(int row = 0; row < 9; row++) {
		const int dy = row % 3 - 1, dz = row / 3 - 1;
		const int *cs = d.cell_start + rp.cell_base + (wrapi(cz + dz, nz) * ny + wrapi(cy + dy, ny)) * nx;
		const int s0 = cs[xa0], e0 = cs[xa1], s1 = inner ? 0 : cs[0], e1 = inner ? 0 : cs[xb1];
		for(int jq = s0; jq < e0; jq++)
			if(jq != i) visit(jq, dy, dz);
		for(int jq = s1; jq < e1; jq++)
			if(jq != i) visit(jq, dy, dz);
	}
}

/* List of sorted position i: the candidates in its 27 cells closer than the replica's list radius. With
 * d.vpairs, also the epoch's flat pair list of the volume pass: every listed candidate above i, one
 * warp-aggregated reservation per warp (at most nl_k per particle, the list's capacity); a particle whose
 * list overflowed goes to vp_over instead and the volume pass scans its half shell in the cells. */
__global__ void __launch_bounds__(NL_B) k_nlist(ppi_dev d) {
	grid_dep_wait(); /* chained by programmatic dependent launch (ppi_resort) */
	grid_dep_release();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = threadIdx.x & 31;
	int n = 0, h = 0, emit = 0, K = d.nl_k, cx = 0, cy = 0, cz = 0, r = 0;
	if(i < d.ntot) {
		const float4 p = d.spos[i];
		const int gc = __float_as_int(d.sori[3 * (size_t) i + 2].z);
		r = d.cell_rep[gc];
		const ppi_rparams &rp = d.rp[r];
		const ppi_grid &g = d.grid[r];
		const float R2 = rp.nl_r2f;
		if(!(R2 > 0.f)) d.nl_cnt[i] = K + 1; /* no lists for this replica: its attempts take the exact path */
		else {
			emit = 1;
			int *out = d.nl + (size_t) i * K;
			const int nx = g.n[0];
			const int local = gc - rp.cell_base;
			cx = local % nx;
			cy = (local / nx) % g.n[1];
			cz = local / (nx * g.n[1]);
			const float wx = g.wf[0], wy = g.wf[1], wz = g.wf[2];
			nl_rows(d, i, rp, g, cx, cy, cz, [&](int jq, int dy, int dz) {
				const float4 q = d.spos[jq];
				int dxc = __float_as_int(q.w) - cx;
				dxc = dxc > 1 ? dxc - nx : (dxc < -1 ? dxc + nx : dxc);
				const float ex = (q.x - p.x) + dxc * wx, ey = (q.y - p.y) + dy * wy, ez = (q.z - p.z) + dz * wz;
				if(fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < R2) {
					if(n < K) out[n] = (int) (((unsigned) jq << 5) | (unsigned) ((dxc + 1) + 3 * (dy + 1) + 9 * (dz + 1)));
					n++;
					h += jq > i;
				}
			});
			d.nl_cnt[i] = n;
			if(n > K) {
				atomicAdd(&d.rs[r].nl_overflow, 1ull);
				h = 0;
				emit = 0;
				if(d.vp_over) d.vp_over[atomicAdd(d.vp_count + 1, 1)] = i;
			}
		}
	}
	if(d.vpairs == nullptr) return;
	int incl = h;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		const int v = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= o) incl += v;
	}
	const int total = __shfl_sync(0xffffffffu, incl, 31);
	int base = 0;
	if(lane == 31 && total) base = atomicAdd(d.vp_count, total);
	base = __shfl_sync(0xffffffffu, base, 31);
	if(!emit || h == 0) return;
	int pos = base + incl - h; /* within capacity: at most nl_k pairs per particle */
	const int *out = d.nl + (size_t) i * K;
	for(int k = 0; k < n; k++) {
		const int e = out[k];
		if((int) ((unsigned) e >> 5) > i) d.vpairs[pos++] = make_int2(i, e);
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* learned proposal                                                                                 */
/* ------------------------------------------------------------------------------------------------ */
/* A learned attempt draws its move from a four-component mixture q(x -> .) = sum_k pi_k(x) K_k, where
 * K_k displaces uniformly in a cube of edge a_k and rotates by an angle uniform in [0, t_k) about a
 * uniform axis (component 0 is the plain move of MC_move_rototranslate, MC.c:311-340: a_0 = Disp_max,
 * t_0 = Theta_max), and pi(x) = (1 - floor) softmax(MLP(features(x))) + floor e_0. The reverse of the
 * move (d, axis, angle) is (-d, -axis, angle): the same |d| and angle, so every K_k has the same density
 * c_k = [|d|_inf <= a_k / 2] [angle < t_k] / (a_k^3 t_k) both ways (relative to a measure common to all
 * components), and Metropolis-Hastings accepts with probability
 *     min(1, exp(-dE / T) sum_k pi_k(x') c_k / sum_k pi_k(x) c_k),     evaluated in FP64.
 * pi is a deterministic function of the particle's canonical state and its neighbours' canonical
 * states: the features read an FP32 image of the FP64 state (simg, computed from rec by explicitly
 * rounded operations), never the FP32 working records. The forward density computed for a move
 * therefore equals the one the reverse move would compute, and the chain keeps the Boltzmann
 * distribution exactly. */
#define TAG_LEARN 7u
#define TAG_COLLECT 8u
#define LEARN_NB 3              /* neighbours in the feature vector (12 patch sites) */
#define PI_BELOW 3.1415925f     /* largest FP32 value below pi: rotation angles stay below pi */
#define LEARN_RF2_SCALE 0.9999f /* feature radius^2 = (1 + delta)^2 (1 - 1e-4): inside the 27 cells */
#define LEARN_LOOSE 1e-3f       /* slack of the working-record pre-filter on r^2 */
#define LIMG 4                  /* float4 per canonical image */
#define LBATCH 4                /* candidates whose loads a lane issues together */

/* Canonical FP32 image of the state (r, q, R0) of particle id: img[0..2] the position wrapped into the
 * box (FP32 guess of the image index, one FP64 operation), img[3] the id, img[4 + 3 i + j] = R_ij of
 * R0 . Q(q / |q|) evaluated in FP32 from the FP32 roundings of q and R0, operation by operation. A
 * deterministic function of the FP64 state; after upload (q the identity) the rows are R0's. */
__device__ __forceinline__ void canon_image(const double *r, const double *q, const double *R0, const double *box, int id, float *img) {
#pragma unroll
	for(int a = 0; a < 3; a++) {
		const float Lf = __double2float_rn(box[a]);
		const float kf = floorf(__fmul_rn(d2f(r[a]), __fdiv_rn(1.f, Lf)));
		img[a] = d2f(__fma_rn(-(double) kf, box[a], r[a]));
	}
	img[3] = __int_as_float(id);
	const float w = d2f(q[0]), x = d2f(q[1]), y = d2f(q[2]), z = d2f(q[3]);
	const float s = __fdiv_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(w, w), __fmul_rn(x, x)), __fadd_rn(__fmul_rn(y, y), __fmul_rn(z, z))));
	float Q[9];
	Q[0] = __fsub_rn(1.f, __fmul_rn(s, __fadd_rn(__fmul_rn(y, y), __fmul_rn(z, z))));
	Q[1] = __fmul_rn(s, __fsub_rn(__fmul_rn(x, y), __fmul_rn(w, z)));
	Q[2] = __fmul_rn(s, __fadd_rn(__fmul_rn(x, z), __fmul_rn(w, y)));
	Q[3] = __fmul_rn(s, __fadd_rn(__fmul_rn(x, y), __fmul_rn(w, z)));
	Q[4] = __fsub_rn(1.f, __fmul_rn(s, __fadd_rn(__fmul_rn(x, x), __fmul_rn(z, z))));
	Q[5] = __fmul_rn(s, __fsub_rn(__fmul_rn(y, z), __fmul_rn(w, x)));
	Q[6] = __fmul_rn(s, __fsub_rn(__fmul_rn(x, z), __fmul_rn(w, y)));
	Q[7] = __fmul_rn(s, __fadd_rn(__fmul_rn(y, z), __fmul_rn(w, x)));
	Q[8] = __fsub_rn(1.f, __fmul_rn(s, __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y))));
#pragma unroll
	for(int i = 0; i < 3; i++) {
		const float a0 = d2f(R0[3 * i]), a1 = d2f(R0[3 * i + 1]), a2 = d2f(R0[3 * i + 2]);
#pragma unroll
		for(int j = 0; j < 3; j++) img[4 + 3 * i + j] = __fadd_rn(__fadd_rn(__fmul_rn(a0, Q[j]), __fmul_rn(a1, Q[3 + j])), __fmul_rn(a2, Q[6 + j]));
	}
	img[13] = img[14] = img[15] = 0.f;
}

__device__ __forceinline__ void load_image(const float4 *simg, int k, float *img) {
#pragma unroll
	for(int c = 0; c < LIMG; c++) {
		const float4 v = simg[LIMG * (size_t) k + c];
		img[4 * c] = v.x, img[4 * c + 1] = v.y, img[4 * c + 2] = v.z, img[4 * c + 3] = v.w;
	}
}

__device__ __forceinline__ void store_image(float4 *simg, int k, const float *img) {
#pragma unroll
	for(int c = 0; c < LIMG; c++) simg[LIMG * (size_t) k + c] = make_float4(img[4 * c], img[4 * c + 1], img[4 * c + 2], img[4 * c + 3]);
}

struct BoxF {
	float L[3], iL[3];
};

__device__ __forceinline__ BoxF box_f(const double *box) {
	BoxF B;
#pragma unroll
	for(int a = 0; a < 3; a++) {
		B.L[a] = __double2float_rn(box[a]);
		B.iL[a] = __fdiv_rn(1.f, B.L[a]);
	}
	return B;
}

__device__ __forceinline__ float min_image(float v, float L, float iL) { return __fsub_rn(v, __fmul_rn(L, rintf(__fmul_rn(v, iL)))); }

/* the up to LEARN_NB nearest neighbours, ordered by (r^2, particle id); pos = sorted position */
struct NbSel {
	float r2[LEARN_NB];
	int key[LEARN_NB];
	int pos[LEARN_NB];
};

__device__ __forceinline__ bool nb_less(float r2a, int ka, float r2b, int kb) { return r2a < r2b || (r2a == r2b && ka < kb); }

__device__ __forceinline__ void nb_clear(NbSel &S) {
#pragma unroll
	for(int n = 0; n < LEARN_NB; n++) {
		S.r2[n] = 3.0e38f;
		S.key[n] = 0x7fffffff;
		S.pos[n] = -1;
	}
}

__device__ __forceinline__ void nb_insert(NbSel &S, float r2, int key, int pos) {
	if(!nb_less(r2, key, S.r2[2], S.key[2])) return;
	S.r2[2] = r2, S.key[2] = key, S.pos[2] = pos;
	if(nb_less(S.r2[2], S.key[2], S.r2[1], S.key[1])) {
		float tr = S.r2[1];
		int tk = S.key[1], tp = S.pos[1];
		S.r2[1] = S.r2[2], S.key[1] = S.key[2], S.pos[1] = S.pos[2];
		S.r2[2] = tr, S.key[2] = tk, S.pos[2] = tp;
		if(nb_less(S.r2[1], S.key[1], S.r2[0], S.key[0])) {
			tr = S.r2[0], tk = S.key[0], tp = S.pos[0];
			S.r2[0] = S.r2[1], S.key[0] = S.key[1], S.pos[0] = S.pos[1];
			S.r2[1] = tr, S.key[1] = tk, S.pos[1] = tp;
		}
	}
}

/* candidate at sorted position k (first float4 of its image: qp) for the feature neighbours of a particle
 * with image pimg: inserted if its canonical distance is below the feature radius. Every kernel decides
 * membership with this function. */
__device__ __forceinline__ void nb_consider(float4 qp, int k, const float *pimg, const BoxF &B, float rf2, NbSel &S) {
	const float vx = min_image(__fsub_rn(qp.x, pimg[0]), B.L[0], B.iL[0]);
	const float vy = min_image(__fsub_rn(qp.y, pimg[1]), B.L[1], B.iL[1]);
	const float vz = min_image(__fsub_rn(qp.z, pimg[2]), B.L[2], B.iL[2]);
	const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
	if(r2 < rf2) nb_insert(S, r2, __float_as_int(qp.w), k);
}

/* the three features of patch site m of a neighbour with image q (centre + 0.5 patch direction, minimum
 * image, relative to the particle with image pimg) in the particle's frame: component c = column c of
 * its orientation . site */
__device__ __forceinline__ void site_feature(const ppi_rparams &rp, const float *pimg, const float *q, int m, const BoxF &B, float *out) {
	float dl[3];
#pragma unroll
	for(int a = 0; a < 3; a++) dl[a] = min_image(__fsub_rn(q[a], pimg[a]), B.L[a], B.iL[a]);
	const float b0 = (float) rp.base[m][0], b1 = (float) rp.base[m][1], b2 = (float) rp.base[m][2];
	float site[3];
#pragma unroll
	for(int a = 0; a < 3; a++) {
		const float p = __fadd_rn(__fadd_rn(__fmul_rn(q[4 + 3 * a], b0), __fmul_rn(q[5 + 3 * a], b1)), __fmul_rn(q[6 + 3 * a], b2));
		site[a] = __fadd_rn(dl[a], __fmul_rn(0.5f, p));
	}
#pragma unroll
	for(int c = 0; c < 3; c++) out[c] = __fadd_rn(__fadd_rn(__fmul_rn(pimg[4 + c], site[0]), __fmul_rn(pimg[7 + c], site[1])), __fmul_rn(pimg[10 + c], site[2]));
}

/* f[12 n + 3 m + c]: patch site m of neighbour n in the particle's frame; zero for absent neighbours */
__device__ __forceinline__ void site_features(const ppi_dev &d, const ppi_rparams &rp, const float *pimg, const NbSel &S, const BoxF &B, float *f) {
	float q[LEARN_NB][16];
#pragma unroll
	for(int n = 0; n < LEARN_NB; n++)
		if(S.pos[n] >= 0) load_image(d.simg, S.pos[n], q[n]); /* the three loads in flight together */
#pragma unroll
	for(int n = 0; n < LEARN_NB; n++)
#pragma unroll
		for(int m = 0; m < 4; m++) {
			if(S.pos[n] >= 0) site_feature(rp, pimg, q[n], m, B, f + 12 * n + 3 * m);
			else f[12 * n + 3 * m] = f[12 * n + 3 * m + 1] = f[12 * n + 3 * m + 2] = 0.f;
		}
}

/* merge the selections of the G lanes of a group (butterfly; every lane ends with the group's result).
 * The order (r^2, id) is total, so the result does not depend on how candidates were split. */
/* The 27 cells around (cx, cy, cz) as one stream of candidates: 9 rows (dy, dz), each the contiguous
 * cells max(cx-1, 0) .. min(cx+1, nx-1) plus the periodic wrap-around cell; range r covers candidates
 * base[r] .. base[r+1]-1 at sorted positions lo[r] + (c - base[r]). The 36 boundary loads are independent. */
struct Cands {
	int lo[18];
	int base[19];
};

__device__ __forceinline__ int cands_build(const ppi_dev &d, const ppi_rparams &rp, const ppi_grid &g, int cx, int cy, int cz, Cands &C) {
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int xa = cx > 0 ? cx - 1 : 0, xb = cx < nx - 1 ? cx + 1 : nx - 1;
	const int xw = cx == 0 ? nx - 1 : (cx == nx - 1 ? 0 : -1);
	int l0[9], h0[9], l1[9], h1[9];
#pragma unroll
	for(int r = 0; r < 9; r++) {
		const int row = rp.cell_base + (wrapi(cz + r / 3 - 1, nz) * ny + wrapi(cy + r % 3 - 1, ny)) * nx;
		l0[r] = d.cell_start[row + xa];
		h0[r] = d.cell_start[row + xb + 1];
		l1[r] = xw >= 0 ? d.cell_start[row + xw] : 0;
		h1[r] = xw >= 0 ? d.cell_start[row + xw + 1] : 0;
	}
	int b = 0;
#pragma unroll
	for(int r = 0; r < 9; r++) {
		C.lo[2 * r] = l0[r];
		C.base[2 * r] = b;
		b += h0[r] - l0[r];
		C.lo[2 * r + 1] = l1[r];
		C.base[2 * r + 1] = b;
		b += h1[r] - l1[r];
	}
	C.base[18] = b;
	return b;
}

/* sorted position of candidate c; the range cursor r only moves forward */
__device__ __forceinline__ int cand_at(const Cands &C, int c, int &r) {
	while(c >= C.base[r + 1]) r++;
	return C.lo[r] + (c - C.base[r]);
}

/* x offset (in cells, -1, 0 or 1) of a candidate in cell column qx seen from column cx */
__device__ __forceinline__ int cell_dx(int qx, int cx, int nx) {
	int v = qx - cx;
	return v > 1 ? v - nx : (v < -1 ? v + nx : v);
}

/* feature neighbours of the particle at sorted position self, cell-local position pl, image pimg: one lane
 * per particle takes candidates sub, sub + 1, ... (sub = 0) */
__device__ __forceinline__ void scan_features(const ppi_dev &d, const ppi_rparams &rp, const ppi_grid &g, const Cands &C, int total, int cx, int self, float4 pl,
		const float *pimg, const BoxF &B, NbSel &S, int sub) {
	constexpr int G = 1; /* candidates a lane skips between its own */
	const float rf2 = __fmul_rn(rp.sqr_rcut_f, LEARN_RF2_SCALE), loose = rf2 + LEARN_LOOSE;
	nb_clear(S);
	int r = 0;
#pragma unroll 1
	for(int c0 = sub; c0 < total; c0 += G * LBATCH) {
		int jq[LBATCH], rr[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			jq[u] = c0 + G * u < total ? cand_at(C, c0 + G * u, r) : -1;
			rr[u] = r >> 1;
		}
		float4 qa[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) qa[u] = jq[u] >= 0 ? d.spos[jq[u]] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
		bool near[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			const float ox = cell_dx(__float_as_int(qa[u].w), cx, g.n[0]) * g.wf[0], oy = (rr[u] % 3 - 1) * g.wf[1], oz = (rr[u] / 3 - 1) * g.wf[2];
			const float ex = (qa[u].x - pl.x) + ox, ey = (qa[u].y - pl.y) + oy, ez = (qa[u].z - pl.z) + oz;
			near[u] = jq[u] >= 0 && jq[u] != self && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < loose;
		}
		float4 qp[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++)
			if(near[u]) qp[u] = d.simg[LIMG * (size_t) jq[u]];
#pragma unroll
		for(int u = 0; u < LBATCH; u++)
			if(near[u]) nb_consider(qp[u], jq[u], pimg, B, rf2, S);
	}
}

/* One scan for the candidate state: bonds of the old (bo) and candidate (bn) state and the feature
 * neighbours of the candidate (image img1) over this lane's candidates sub, sub + 1, ... False if one of
 * them overlaps the candidate state. */
template <int MODE>
__device__ __forceinline__ bool scan_move(const ppi_dev &d, const Proposal &P, const Cands &C, int total, int cx, const float *cpn, const float *img1, const BoxF &B,
		NbSel &S, int &bo, int &bn, Acc &A, int sub) {
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	ppi_rstate *rs = d.rs + P.r;
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float rc2e = rp.sqr_rcut_f + eps, ovl = 1.f - eps;
	const float rf2 = __fmul_rn(rp.sqr_rcut_f, LEARN_RF2_SCALE), loose = rf2 + LEARN_LOOSE;
	const float4 pn = make_float4(P.po.x + P.disp.x, P.po.y + P.disp.y, P.po.z + P.disp.z, 0.f);
	constexpr int G = 1; /* candidates a lane skips between its own */
	nb_clear(S);
	bo = bn = 0;
	int r = 0;
#pragma unroll 1
	for(int c0 = sub; c0 < total; c0 += G * LBATCH) {
		int jq[LBATCH], rr[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			jq[u] = c0 + G * u < total ? cand_at(C, c0 + G * u, r) : -1;
			rr[u] = r >> 1;
		}
		float4 qa[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) qa[u] = jq[u] >= 0 ? d.spos[jq[u]] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
		float go[LBATCH][3], gn[LBATCH][3];
		bool feat[LBATCH], pair[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			const float ox = cell_dx(__float_as_int(qa[u].w), cx, g.n[0]) * g.wf[0], oy = (rr[u] % 3 - 1) * g.wf[1], oz = (rr[u] / 3 - 1) * g.wf[2];
			go[u][0] = (qa[u].x - P.po.x) + ox, go[u][1] = (qa[u].y - P.po.y) + oy, go[u][2] = (qa[u].z - P.po.z) + oz;
			gn[u][0] = (qa[u].x - pn.x) + ox, gn[u][1] = (qa[u].y - pn.y) + oy, gn[u][2] = (qa[u].z - pn.z) + oz;
			const float r2o = fmaf(go[u][0], go[u][0], fmaf(go[u][1], go[u][1], go[u][2] * go[u][2]));
			const float r2n = fmaf(gn[u][0], gn[u][0], fmaf(gn[u][1], gn[u][1], gn[u][2] * gn[u][2]));
			const bool live = jq[u] >= 0 && jq[u] != P.i;
			if(live) A.pairs += 2;
			if(MODE != MODE_AUDIT && live && r2n < ovl) return false;
			feat[u] = live && r2n < loose;
			pair[u] = live && (MODE == MODE_AUDIT || r2o < rc2e || r2n < rc2e);
		}
		float4 qp[LBATCH], qb[LBATCH], qc[LBATCH], qd[LBATCH];
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			if(feat[u]) qp[u] = d.simg[LIMG * (size_t) jq[u]];
			if(pair[u]) {
				qb[u] = d.sori[3 * (size_t) jq[u]];
				qc[u] = d.sori[3 * (size_t) jq[u] + 1];
				qd[u] = d.sori[3 * (size_t) jq[u] + 2];
			}
		}
#pragma unroll
		for(int u = 0; u < LBATCH; u++) {
			if(feat[u]) nb_consider(qp[u], jq[u], img1, B, rf2, S);
			if(!pair[u]) continue;
			const float cq[9] = { qb[u].x, qb[u].y, qb[u].z, qb[u].w, qc[u].x, qc[u].y, qc[u].z, qc[u].w, qd[u].x };
			const int qslot = __float_as_int(qd[u].w);
			const int clo = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 0, P.q, P.disp, qslot, go[u][0], go[u][1], go[u][2], P.cpo, cq, rp.sqr_rcut_f, rp.cosmax_f,
					rp.base_f, eps, 0, nullptr, nullptr, A.fallbacks);
			const int cln = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 1, P.q, P.disp, qslot, gn[u][0], gn[u][1], gn[u][2], cpn, cq, rp.sqr_rcut_f, rp.cosmax_f,
					rp.base_f, eps, 0, nullptr, nullptr, A.fallbacks);
			if(cln == CL_OVER) return false;
			bo += (clo == CL_BOND);
			bn += (cln == CL_BOND);
		}
	}
	return true;
}

/* move of component k from two Philox blocks: displacement (rd.x, rd.y, rd.z), angle rd.w, axis (ra.x, ra.y);
 * component 0 reproduces the plain move's arithmetic */
__device__ __forceinline__ void mix_draw(float a, float t, U4 rd, U4 ra, float3 &disp, float &theta, float4 &q) {
	disp = make_float3((u01(rd.x) - 0.5f) * a, (u01(rd.y) - 0.5f) * a, (u01(rd.z) - 0.5f) * a);
	theta = u01(rd.w) * t;
	const float zc = 1.f - 2.f * u01(ra.x);
	const float phi = 6.283185307179586f * u01(ra.y);
	const float sr = sqrtf(fmaxf(0.f, 1.f - zc * zc));
	float sp, cph, sh, ch;
	__sincosf(phi, &sp, &cph);
	__sincosf(0.5f * theta, &sh, &ch);
	q = make_float4(ch, sh * sr * cph, sh * sr * sp, sh * zc);
}

/* sum_k pi_k c_k of a move (FP64; the component densities of the replica precomputed, ppi_lrep) */
__device__ __forceinline__ double mix_density(const float *pi, const ppi_lrep &M, float3 dsp, float theta) {
	const float m = fmaxf(fabsf(dsp.x), fmaxf(fabsf(dsp.y), fabsf(dsp.z)));
	double s = 0.;
#pragma unroll
	for(int k = 0; k < PPI_MIX; k++)
		if(m <= 0.5f * M.a[k] && theta < M.t[k]) s = fma((double) pi[k], M.v[k], s);
	return s;
}

/* canonical state of the mover after the move (dq, disp): commit_move's FP64 operations, then its image */
__device__ __forceinline__ void moved_image(const double *rec, int id, float4 dq, float3 disp, const double *box, float *img) {
	const double qv[4] = { rec[PPI_Q], rec[PPI_Q + 1], rec[PPI_Q + 2], rec[PPI_Q + 3] };
	const double b[4] = { f2d(dq.x), f2d(dq.y), f2d(dq.z), f2d(dq.w) };
	double qn[4], R0[9];
#pragma unroll
	for(int c = 0; c < 4; c++) qn[c] = qcomp64(qv[c], qv[c ^ 1], qv[c ^ 2], qv[c ^ 3], b, c);
	const double rn[3] = { __dadd_rn(rec[0], f2d(disp.x)), __dadd_rn(rec[1], f2d(disp.y)), __dadd_rn(rec[2], f2d(disp.z)) };
#pragma unroll
	for(int k = 0; k < 9; k++) R0[k] = rec[PPI_R0 + k];
	canon_image(rn, qn, R0, box, id, img);
}

/* the mover of a list entry: particle choice (draw), working record, canonical image, cell */
__device__ __forceinline__ void learn_mover(const ppi_dev &d, const int4 ent, uint32_t draw, Proposal &P, float *img, int &cx, int &cy, int &cz) {
	P.r = ent.w;
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	P.local = ent.x - rp.cell_base;
	P.i = ent.y + (int) __umulhi(draw, (uint32_t) ent.z);
	P.po = d.spos[P.i];
	const float4 ob = d.sori[3 * (size_t) P.i], oc = d.sori[3 * (size_t) P.i + 1], od = d.sori[3 * (size_t) P.i + 2];
	load_image(d.simg, P.i, img);
	P.pslot = __float_as_int(od.w);
	P.cpo[0] = ob.x, P.cpo[1] = ob.y, P.cpo[2] = ob.z, P.cpo[3] = ob.w;
	P.cpo[4] = oc.x, P.cpo[5] = oc.y, P.cpo[6] = oc.z, P.cpo[7] = oc.w;
	P.cpo[8] = od.x;
	cx = P.local % g.n[0];
	cy = (P.local / g.n[0]) % g.n[1];
	cz = P.local / (g.n[0] * g.n[1]);
}

__device__ __forceinline__ bool inside_cell(const ppi_grid &g, float4 po, float3 disp) {
	const float nx = po.x + disp.x, ny = po.y + disp.y, nz = po.z + disp.z;
	return nx >= 0.f && nx < g.wf[0] && ny >= 0.f && ny < g.wf[1] && nz >= 0.f && nz < g.wf[2];
}

/* warp-wide flush of the per-lane counters (one atomic per counter when the lanes share a replica) */
__device__ __forceinline__ void flush_warp(const ppi_dev &d, Acc &A) {
	const unsigned same = __match_any_sync(0xffffffffu, A.r);
	if(same != 0xffffffffu || A.r < 0) {
		flush_thread(d, A);
		return;
	}
	const unsigned t = __reduce_add_sync(0xffffffffu, A.tries), ac = __reduce_add_sync(0xffffffffu, A.acc);
	const unsigned p = __reduce_add_sync(0xffffffffu, A.pairs), f = __reduce_add_sync(0xffffffffu, A.fallbacks);
	const int db = __reduce_add_sync(0xffffffffu, A.dbonds);
	if((threadIdx.x & 31) == 0) {
		ppi_rstate *rs = d.rs + A.r;
		if(t) atomicAdd(&rs->tries[0], (unsigned long long) t);
		if(ac) atomicAdd(&rs->accepted[0], (unsigned long long) ac);
		if(p) atomicAdd(&rs->pairs, (unsigned long long) p);
		if(f) atomicAdd(&rs->fallbacks, (unsigned long long) f);
		if(db) atomicAdd((unsigned long long *) &rs->bonds, (unsigned long long) (long long) db);
	}
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
}

/* Per-lane candidate cache of the learned colour kernel (shared memory, [slot][lane] so that a warp's
 * accesses to one slot are conflict-free): the scans gather the working-record positions of up to LCAP
 * candidates, then the canonical positions of the close ones and the orientations of the bonding-range
 * ones, each batch with asynchronous copies that are all in flight together (one memory latency per
 * batch instead of one per candidate). */
#define LCAP 16
#define LPB 4 /* pairs per orientation batch */
#define LEARN_CACHE_OFF ((sizeof(MlpWarpSmem) + 127) / 128 * 128)
#define LEARN_SMEM (LEARN_CACHE_OFF + sizeof(LearnCache))
struct __align__(16) LearnCache {
	float4 pos[LCAP][32];
	float4 img[LCAP][LIMG][32]; /* canonical images of the close candidates */
	float4 ori[LPB][3][32];
	double2 rec[PPI_REC / 2][32]; /* the mover's FP64 record */
	int jq[LCAP][32];             /* sorted position << 4 | row (0..8) */
};

/* all four float4 of the canonical image of sorted position jq into cache slot k */
__device__ __forceinline__ void cache_image(const ppi_dev &d, LearnCache &K, int k, int jq) {
	const int l = threadIdx.x;
#pragma unroll
	for(int c = 0; c < LIMG; c++) cp_async16(&K.img[k][c][l], d.simg + LIMG * (size_t) jq + c);
}

/* features from the images the scan left in the cache (ncached candidates of its last chunk); a
 * neighbour outside it (scans of more than LCAP candidates) is read from global memory */
__device__ __forceinline__ void site_features_cached(const ppi_dev &d, const LearnCache &K, int ncached, const ppi_rparams &rp, const float *pimg, const NbSel &S, const BoxF &B,
		float *f) {
	const int l = threadIdx.x;
#pragma unroll
	for(int n = 0; n < LEARN_NB; n++) {
		if(S.pos[n] < 0) {
#pragma unroll
			for(int e = 0; e < 12; e++) f[12 * n + e] = 0.f;
			continue;
		}
		int slot = -1;
		for(int k = 0; k < ncached; k++)
			if((K.jq[k][l] >> 4) == S.pos[n]) {
				slot = k;
				break;
			}
		float q[16];
		if(slot >= 0) {
#pragma unroll
			for(int c = 0; c < LIMG; c++) {
				const float4 v = K.img[slot][c][l];
				q[4 * c] = v.x, q[4 * c + 1] = v.y, q[4 * c + 2] = v.z, q[4 * c + 3] = v.w;
			}
		}
		else load_image(d.simg, S.pos[n], q);
#pragma unroll
		for(int m = 0; m < 4; m++) site_feature(rp, pimg, q, m, B, f + 12 * n + 3 * m);
	}
}

/* gathers the working-record positions of candidates c0 .. c0 + n - 1 of this lane */
__device__ __forceinline__ void cache_positions(const ppi_dev &d, LearnCache &K, const Cands &C, int c0, int n, int &r) {
	const int l = threadIdx.x;
	for(int k = 0; k < n; k++) {
		const int jq = cand_at(C, c0 + k, r);
		K.jq[k][l] = (jq << 4) | (r >> 1);
		cp_async16(&K.pos[k][l], d.spos + jq);
	}
	cp_async_wait_all();
}

/* feature neighbours of the current state from the cache (see scan_features) */
__device__ __forceinline__ int scan_features_cached(const ppi_dev &d, LearnCache &K, const ppi_rparams &rp, const ppi_grid &g, const Cands &C, int total, int cx, int self,
		float4 pl, const float *pimg, const BoxF &B, NbSel &S, int *ncached) {
	const int l = threadIdx.x;
	const float rf2 = __fmul_rn(rp.sqr_rcut_f, LEARN_RF2_SCALE), loose = rf2 + LEARN_LOOSE;
	nb_clear(S);
	int r = 0, last = 0;
	for(int c0 = 0; c0 < total; c0 += LCAP) {
		const int n = min(LCAP, total - c0);
		cache_positions(d, K, C, c0, n, r);
		last = n;
		unsigned near = 0u;
		for(int k = 0; k < n; k++) {
			const float4 qa = K.pos[k][l];
			const int e = K.jq[k][l], jq = e >> 4, rr = e & 15;
			const float ox = cell_dx(__float_as_int(qa.w), cx, g.n[0]) * g.wf[0], oy = (rr % 3 - 1) * g.wf[1], oz = (rr / 3 - 1) * g.wf[2];
			const float ex = (qa.x - pl.x) + ox, ey = (qa.y - pl.y) + oy, ez = (qa.z - pl.z) + oz;
			if(jq != self && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < loose) {
				near |= 1u << k;
				cache_image(d, K, k, jq);
			}
		}
		cp_async_wait_all();
		while(near) {
			const int k = __ffs(near) - 1;
			near &= near - 1u;
			nb_consider(K.img[k][0][l], K.jq[k][l] >> 4, pimg, B, rf2, S);
		}
	}
	*ncached = last;
	return total <= LCAP ? last : -1; /* candidates still in the cache (all of them), or -1 */
}

/* bonds of the old and candidate state and the candidate's feature neighbours from the cache (see
 * scan_move); cached = number of candidates the feature scan left in the cache (-1: reload) */
template <int MODE>
__device__ __forceinline__ bool scan_move_cached(const ppi_dev &d, LearnCache &K, const Proposal &P, const Cands &C, int total, int cached, int cx, const float *cpn,
		const float *img1, const BoxF &B, NbSel &S, int &bo, int &bn, Acc &A, int *ncached) {
	const int l = threadIdx.x;
	const ppi_rparams &rp = d.rp[P.r];
	const ppi_grid &g = d.grid[P.r];
	ppi_rstate *rs = d.rs + P.r;
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float rc2e = rp.sqr_rcut_f + eps, ovl = 1.f - eps;
	const float rf2 = __fmul_rn(rp.sqr_rcut_f, LEARN_RF2_SCALE), loose = rf2 + LEARN_LOOSE;
	const float4 pn = make_float4(P.po.x + P.disp.x, P.po.y + P.disp.y, P.po.z + P.disp.z, 0.f);
	nb_clear(S);
	bo = bn = 0;
	int r = 0;
	*ncached = 0;
	for(int c0 = 0; c0 < total; c0 += LCAP) {
		const int n = min(LCAP, total - c0);
		if(cached < 0) cache_positions(d, K, C, c0, n, r);
		*ncached = n;
		unsigned feat = 0u, pair = 0u;
		for(int k = 0; k < n; k++) {
			const float4 qa = K.pos[k][l];
			const int e = K.jq[k][l], jq = e >> 4, rr = e & 15;
			if(jq == P.i) continue;
			const float ox = cell_dx(__float_as_int(qa.w), cx, g.n[0]) * g.wf[0], oy = (rr % 3 - 1) * g.wf[1], oz = (rr / 3 - 1) * g.wf[2];
			const float dxo = (qa.x - P.po.x) + ox, dyo = (qa.y - P.po.y) + oy, dzo = (qa.z - P.po.z) + oz;
			const float dxn = (qa.x - pn.x) + ox, dyn = (qa.y - pn.y) + oy, dzn = (qa.z - pn.z) + oz;
			const float r2o = fmaf(dxo, dxo, fmaf(dyo, dyo, dzo * dzo)), r2n = fmaf(dxn, dxn, fmaf(dyn, dyn, dzn * dzn));
			A.pairs += 2;
			if(MODE != MODE_AUDIT && r2n < ovl) {
				cp_async_wait_all();
				return false;
			}
			if(r2n < loose) {
				feat |= 1u << k;
				cache_image(d, K, k, jq);
			}
			if(MODE == MODE_AUDIT || r2o < rc2e || r2n < rc2e) pair |= 1u << k;
		}
		cp_async_wait_all();
		while(feat) {
			const int k = __ffs(feat) - 1;
			feat &= feat - 1u;
			nb_consider(K.img[k][0][l], K.jq[k][l] >> 4, img1, B, rf2, S);
		}
		/* pair tests, LPB orientation gathers in flight at a time */
		while(pair) {
			int ks[LPB], nb = 0;
			while(pair && nb < LPB) {
				ks[nb] = __ffs(pair) - 1;
				pair &= pair - 1u;
				const int jq = K.jq[ks[nb]][l] >> 4;
#pragma unroll
				for(int c = 0; c < 3; c++) cp_async16(&K.ori[nb][c][l], d.sori + 3 * (size_t) jq + c);
				nb++;
			}
			cp_async_wait_all();
			for(int b = 0; b < nb; b++) {
				const int k = ks[b];
				const float4 qa = K.pos[k][l];
				const int rr = K.jq[k][l] & 15;
				const float ox = cell_dx(__float_as_int(qa.w), cx, g.n[0]) * g.wf[0], oy = (rr % 3 - 1) * g.wf[1], oz = (rr / 3 - 1) * g.wf[2];
				const float dxo = (qa.x - P.po.x) + ox, dyo = (qa.y - P.po.y) + oy, dzo = (qa.z - P.po.z) + oz;
				const float dxn = (qa.x - pn.x) + ox, dyn = (qa.y - pn.y) + oy, dzn = (qa.z - pn.z) + oz;
				const float4 qb = K.ori[b][0][l], qc = K.ori[b][1][l], qd = K.ori[b][2][l];
				const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
				const int qslot = __float_as_int(qd.w);
				const int clo = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 0, P.q, P.disp, qslot, dxo, dyo, dzo, P.cpo, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr,
						nullptr, A.fallbacks);
				const int cln = pair_state<MODE>(d.rec, rp, rs, g.inv_L, P.pslot, 1, P.q, P.disp, qslot, dxn, dyn, dzn, cpn, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, 0, nullptr, nullptr,
						A.fallbacks);
				if(cln == CL_OVER) return false;
				bo += (clo == CL_BOND);
				bn += (cln == CL_BOND);
			}
		}
	}
	return true;
}

/* One checkerboard colour of learned moves: one warp per CTA, 32 attempts per tile (one per lane); the
 * network runs twice per tile on the tensor cores (current and candidate states). */
template <int MODE>
__global__ void __launch_bounds__(32) k_colour_learned(ppi_dev d, long long round, int col) {
	if(round < 0) { /* graph launch (see k_colour) */
		round = ctr_index(round, d.ctr->round);
		col = colour_at(round, col);
	}
	const int4 *list = d.clist + (size_t) col * d.clist_cap;
	int cnt = d.ccount[col];
	if(cnt > d.clist_cap) cnt = d.clist_cap;
	const int ntiles = (cnt + 31) / 32;
	if((int) blockIdx.x >= ntiles) return; /* the whole CTA: no tensor memory taken */
	extern __shared__ __align__(128) unsigned char smem_raw[];
	MlpWarpSmem &S = *(MlpWarpSmem *) smem_raw;
	LearnCache &K = *(LearnCache *) (smem_raw + LEARN_CACHE_OFF);
	mlpw_begin(S, d.mlp_img);
	const ppi_learn L = *d.learn;
	uint32_t phase = 0;
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	unsigned ctr[PPI_MIX] = { 0u, 0u, 0u, 0u }, cac[PPI_MIX] = { 0u, 0u, 0u, 0u };
	bool waited = false;
#pragma unroll 1
	for(int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		const int idx = tile * 32 + threadIdx.x;
		bool live = idx < cnt;
		Proposal P;
		P.r = 0;
		float img0[16], f[MLP_IN];
		int cx = 0, cy = 0, cz = 0, total = 0, cached = -1;
		U4 r1 = U4{ 0u, 0u, 0u, 0u };
		Cands C;
#pragma unroll
		for(int e = 0; e < MLP_IN; e++) f[e] = 0.f;
		if(live) {
			/* what reads only the mover, the epoch's cell ranges and the network: before the wait on the
			 * previous colour (programmatic dependent launch, see grid_dep_wait) */
			const int4 ent = list[idx];
			const ppi_rparams &rp = d.rp[ent.w];
			r1 = rng(rp, round, ent.w, TAG_LEARN, (uint32_t) (ent.x - rp.cell_base), 0u);
			learn_mover(d, ent, r1.x, P, img0, cx, cy, cz);
			total = cands_build(d, rp, d.grid[P.r], cx, cy, cz, C);
			/* the mover's FP64 record, in flight while the features are formed */
#pragma unroll
			for(int c = 0; c < PPI_REC / 2; c++) cp_async16(&K.rec[c][threadIdx.x], d.rec + (size_t) P.pslot * PPI_REC + 2 * c);
		}
		if(!waited) {
			grid_dep_wait();
			grid_dep_release();
			waited = true;
		}
		if(live) {
			const ppi_rparams &rp = d.rp[P.r];
			if(P.r != A.r) {
				flush_thread(d, A);
				A.r = P.r;
			}
			A.tries++;
			const ppi_grid &g = d.grid[P.r];
			const BoxF B = box_f(d.rs[P.r].box);
			NbSel sel;
			int nc = 0;
			cached = scan_features_cached(d, K, rp, g, C, total, cx, P.i, P.po, img0, B, sel, &nc);
			site_features_cached(d, K, nc, rp, img0, sel, B, f);
		}
		mlpw_put_x(S, f);
		float z[MLP_OUT], pi0[PPI_MIX], pi1[PPI_MIX];
		mlpw_forward(S, &phase, z);
		mix_weights(z, L.floor0, pi0);
		int comp = 0, bo = 0, bn = 0;
		float theta = 0.f, img1[16], cpn[9];
		double recl[PPI_REC];
#pragma unroll
		for(int e = 0; e < MLP_IN; e++) f[e] = 0.f;
		if(live) {
			const ppi_rparams &rp = d.rp[P.r];
			const ppi_lrep &M = d.lrep[P.r];
			const float uc = u01(r1.y);
			float cum = pi0[0];
			while(comp < PPI_MIX - 1 && uc >= cum) cum = __fadd_rn(cum, pi0[++comp]);
			const U4 rd = rng(rp, round, P.r, TAG_LEARN, (uint32_t) P.local, 1u), ra = rng(rp, round, P.r, TAG_LEARN, (uint32_t) P.local, 2u);
			mix_draw(M.a[comp], M.t[comp], rd, ra, P.disp, theta, P.q);
			ctr[comp]++;
			live = inside_cell(d.grid[P.r], P.po, P.disp);
			if(live) {
				const BoxF B = box_f(d.rs[P.r].box);
				cp_async_wait_all();
#pragma unroll
				for(int c = 0; c < PPI_REC / 2; c++) {
					const double2 v = K.rec[c][threadIdx.x];
					recl[2 * c] = v.x;
					recl[2 * c + 1] = v.y;
				}
				moved_image(recl, __float_as_int(img0[3]), P.q, P.disp, d.rs[P.r].box, img1);
				cols_new(P.cpo, P.q, cpn);
				NbSel sel;
				int nc = 0;
				live = scan_move_cached<MODE>(d, K, P, C, total, cached, cx, cpn, img1, B, sel, bo, bn, A, &nc);
				if(live) site_features_cached(d, K, nc, rp, img1, sel, B, f);
			}
		}
		mlpw_put_x(S, f);
		mlpw_forward(S, &phase, z);
		mix_weights(z, L.floor0, pi1);
		if(live) {
			const ppi_lrep &M = d.lrep[P.r];
			const int dE = bo - bn;
			const double bz = (dE >= -PPI_LEXP && dE <= PPI_LEXP) ? M.expk[dE + PPI_LEXP] : exp(-(double) dE / d.rp[P.r].T);
			/* accept iff U < exp(-dE / T) q(x' -> x) / q(x -> x'), without the division */
			if(u01d(r1.z, r1.w) * mix_density(pi0, M, P.disp, theta) < bz * mix_density(pi1, M, P.disp, theta)) {
				commit_from(d, recl, P.i, P.pslot, P.po, P.disp, P.q, cpn);
				store_image(d.simg, P.i, img1);
				A.acc++;
				A.dbonds += bn - bo;
				cac[comp]++;
			}
		}
		cp_async_wait_all(); /* no copy of this tile may land in the next tile's buffers */
	}
	flush_warp(d, A);
#pragma unroll
	for(int k = 0; k < PPI_MIX; k++) {
		const unsigned tk = __reduce_add_sync(0xffffffffu, ctr[k]), ak = __reduce_add_sync(0xffffffffu, cac[k]);
		if(threadIdx.x == 0 && tk) {
			atomicAdd(d.lstats + k, (unsigned long long) tk);
			if(ak) atomicAdd(d.lstats + PPI_MIX + k, (unsigned long long) ak);
		}
	}
	mlpw_end(S);
	if(threadIdx.x == 0 && S.err) atomicExch(d.lerr, 1);
}

/* Training samples of the current state: row j of [base, base + count) takes list entry j * n / count of
 * colour col, its particle's features and, per component k, the mean over `draws` proposals of
 *     u_k = kappa |bonds_new - bonds_old| min(1, exp(-(dE - 1) / T)) + jump acc (|d|^2 / Disp_max^2 + angle^2 / Theta_max^2)
 * for a candidate inside the cell without overlap (else 0), acc = min(1, exp(-dE / T)). The first term
 * counts proposals that change the particle's bond count, weighted by their acceptance relative to that
 * of breaking one bond: in a bonded network bond turnover is limited by breaking, which every component
 * accepts with the same exp(-1 / T), so what a component adds is how often it proposes one. The second is
 * a tie-break for particles without partners in reach (acceptance-weighted squared jump). The four
 * utilities are stored divided by the largest. */
template <int MODE>
__global__ void __launch_bounds__(128) k_learn_collect(ppi_dev d, long long snap, int col, int base, int count) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= count) return;
	float *out = d.samples + (size_t) (base + j) * MLP_SAMPLE;
	int cnt = d.ccount[col];
	if(cnt > d.clist_cap) cnt = d.clist_cap;
	if(cnt == 0) {
		for(int e = 0; e < MLP_SAMPLE; e++) out[e] = 0.f;
		return;
	}
	const ppi_learn L = *d.learn;
	const int4 ent = d.clist[(size_t) col * d.clist_cap + (int) (((long long) j * cnt) / count)];
	const ppi_rparams &rp = d.rp[ent.w];
	const ppi_lrep &M = d.lrep[ent.w];
	const U4 r1 = rng(rp, snap, ent.w, TAG_COLLECT, (uint32_t) (ent.x - rp.cell_base), 0u);
	Proposal P;
	float img0[16], f[MLP_IN];
	int cx, cy, cz;
	learn_mover(d, ent, r1.x, P, img0, cx, cy, cz);
	const ppi_grid &g = d.grid[P.r];
	Cands C;
	const int total = cands_build(d, rp, g, cx, cy, cz, C);
	const BoxF B = box_f(d.rs[P.r].box);
	NbSel sel;
	scan_features(d, rp, g, C, total, cx, P.i, P.po, img0, B, sel, 0);
	site_features(d, rp, img0, sel, B, f);
#pragma unroll
	for(int e = 0; e < MLP_IN; e++) out[e] = f[e];
	const float idm2 = 1.f / (rp.disp_max_f * rp.disp_max_f), ith2 = 1.f / (rp.theta_max_f * rp.theta_max_f);
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	float uk[PPI_MIX];
	float img1[16];
#pragma unroll 1
	for(int k = 0; k < PPI_MIX; k++) {
		float u = 0.f;
#pragma unroll 1
		for(int q = 0; q < L.draws; q++) {
			const uint32_t sub = 1u + 2u * (uint32_t) (k * L.draws + q);
			const U4 rd = rng(rp, snap, P.r, TAG_COLLECT, (uint32_t) P.local, sub), ra = rng(rp, snap, P.r, TAG_COLLECT, (uint32_t) P.local, sub + 1u);
			float theta;
			mix_draw(M.a[k], M.t[k], rd, ra, P.disp, theta, P.q);
			if(!inside_cell(g, P.po, P.disp)) continue;
			float cpn[9];
			cols_new(P.cpo, P.q, cpn);
			int bo, bn;
			NbSel s2;
			img1[0] = img1[1] = img1[2] = 0.f; /* the candidate's features are not needed here */
			if(!scan_move<MODE>(d, P, C, total, cx, cpn, img1, B, s2, bo, bn, A, 0)) continue;
			const int dE = bo - bn;
			const float acc = dE <= 0 ? 1.f : (float) ((dE <= PPI_LEXP) ? M.expk[dE + PPI_LEXP] : exp(-(double) dE / rp.T));
			const float acc1 = dE <= 1 ? 1.f : (float) ((dE - 1 <= PPI_LEXP) ? M.expk[dE - 1 + PPI_LEXP] : exp(-(double) (dE - 1) / rp.T));
			const float d2 = P.disp.x * P.disp.x + P.disp.y * P.disp.y + P.disp.z * P.disp.z;
			u += L.kappa * (float) abs(bn - bo) * acc1 + L.jump * acc * (d2 * idm2 + theta * theta * ith2);
		}
		uk[k] = u / (float) L.draws;
	}
	const float um = fmaxf(fmaxf(uk[0], uk[1]), fmaxf(uk[2], uk[3]));
#pragma unroll
	for(int k = 0; k < PPI_MIX; k++) out[MLP_IN + k] = um > 0.f ? uk[k] / um : 0.f;
}

/* features of the particle at every sorted position, stored by slot (d.feat[slot][36]) */
__global__ void k_learn_features(ppi_dev d) {
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= d.ntot) return;
	const float4 od = d.sori[3 * (size_t) k + 2];
	const int gc = __float_as_int(od.z), slot = __float_as_int(od.w);
	const int r = d.cell_rep[gc];
	const ppi_rparams &rp = d.rp[r];
	const ppi_grid &g = d.grid[r];
	const int local = gc - rp.cell_base;
	const int cx = local % g.n[0], cy = (local / g.n[0]) % g.n[1], cz = local / (g.n[0] * g.n[1]);
	const float4 po = d.spos[k];
	float img[16], f[MLP_IN];
	load_image(d.simg, k, img);
	const BoxF B = box_f(d.rs[r].box);
	Cands C;
	const int total = cands_build(d, rp, g, cx, cy, cz, C);
	NbSel sel;
	scan_features(d, rp, g, C, total, cx, k, po, img, B, sel, 0);
	site_features(d, rp, img, sel, B, f);
	for(int e = 0; e < MLP_IN; e++) d.feat[(size_t) slot * MLP_IN + e] = f[e];
}

/* canonical images of every sorted position from the FP64 records and the current boxes */
__global__ void k_canon(ppi_dev d) {
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= d.ntot) return;
	const int s = __float_as_int(d.sori[3 * (size_t) k + 2].w);
	const double *rec = d.rec + (size_t) s * PPI_REC;
	double q[4], R0[9];
	const double r[3] = { rec[0], rec[1], rec[2] };
#pragma unroll
	for(int c = 0; c < 4; c++) q[c] = rec[PPI_Q + c];
#pragma unroll
	for(int j = 0; j < 9; j++) R0[j] = rec[PPI_R0 + j];
	float img[16];
	canon_image(r, q, R0, d.rs[d.rep[s]].box, d.id[s], img);
	store_image(d.simg, k, img);
}

/* ------------------------------------------------------------------------------------------------ */
/* lane groups (energy pass)                                                                        */
/* ------------------------------------------------------------------------------------------------ */
#define PPI_DEFAULT_LANES 4
template <int G>
__device__ __forceinline__ unsigned group_mask() {
	if(G >= 32) return 0xffffffffu;
	return ((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1));
}

template <int G>
__device__ __forceinline__ int group_sum(unsigned gm, int v) {
#pragma unroll
	for(int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o);
	return v;
}

/* ------------------------------------------------------------------------------------------------ */
/* energy from scratch: bonds / overlaps per particle, or the NPT candidate box                     */
/* ------------------------------------------------------------------------------------------------ */
/* energy pass counters: bonds in A.tries (summed into rs.vol_bonds), pairs, fallbacks */
__device__ __forceinline__ void energy_flush_thread(const ppi_dev &d, Acc &A) {
	if(A.r < 0) return;
	ppi_rstate *rs = d.rs + A.r;
	if(A.tries) atomicAdd((unsigned long long *) &rs->vol_bonds, (unsigned long long) A.tries);
	if(A.pairs) atomicAdd(&rs->pairs, (unsigned long long) A.pairs);
	if(A.fallbacks) atomicAdd(&rs->fallbacks, (unsigned long long) A.fallbacks);
	A.tries = A.pairs = A.fallbacks = 0;
}

__device__ __forceinline__ void energy_flush_block(const ppi_dev &d, Acc &A) {
	__shared__ int s_rep, s_mixed;
	__shared__ unsigned s_v[3];
	if(threadIdx.x == 0) {
		s_rep = -1;
		s_mixed = 0;
		s_v[0] = s_v[1] = s_v[2] = 0;
	}
	__syncthreads();
	if(A.r >= 0) {
		int old = atomicCAS(&s_rep, -1, A.r);
		if(old != -1 && old != A.r) s_mixed = 1;
	}
	__syncthreads();
	if(s_mixed) {
		energy_flush_thread(d, A);
		return;
	}
	unsigned b = __reduce_add_sync(0xffffffffu, A.tries), p = __reduce_add_sync(0xffffffffu, A.pairs), f = __reduce_add_sync(0xffffffffu, A.fallbacks);
	if((threadIdx.x & 31) == 0) {
		atomicAdd(&s_v[0], b);
		atomicAdd(&s_v[1], p);
		atomicAdd(&s_v[2], f);
	}
	__syncthreads();
	if(threadIdx.x == 0 && s_rep >= 0) {
		ppi_rstate *rs = d.rs + s_rep;
		if(s_v[0]) atomicAdd((unsigned long long *) &rs->vol_bonds, (unsigned long long) s_v[0]);
		if(s_v[1]) atomicAdd(&rs->pairs, (unsigned long long) s_v[1]);
		if(s_v[2]) atomicAdd(&rs->fallbacks, (unsigned long long) s_v[2]);
	}
}

/* energy of particle k (sorted position) on its own, every guard-band pair decided exactly on the spot
 * (the deferred particles of the energy pass) */
__device__ __forceinline__ void energy_exact(const ppi_dev &d, int mode, int k, Acc &A) {
	const float4 pa = d.spos[k], pb = d.sori[3 * (size_t) k], pc = d.sori[3 * (size_t) k + 1], pd = d.sori[3 * (size_t) k + 2];
	const int gc = __float_as_int(pd.z);
	const int r = d.cell_rep[gc];
	if(r != A.r) {
		energy_flush_thread(d, A);
		A.r = r;
	}
	const ppi_rparams &rp = d.rp[r];
	const ppi_grid &g = d.grid[r];
	ppi_rstate *rs = d.rs + r;
	int vmask = 0;
	float sf3[3] = { 1.f, 1.f, 1.f };
	const double *vf3 = nullptr, *vb3 = nullptr;
	if(mode == PPI_EN_VOLUME) {
		if(g.vol_dir < 0 || rs->vol_overlap) return;
		vmask = g.vol_mask;
		sf3[0] = g.vol_ff3[0];
		sf3[1] = g.vol_ff3[1];
		sf3[2] = g.vol_ff3[2];
		vf3 = g.vol_f3;
		vb3 = g.vol_box3;
	}
	float w[3] = { g.wf[0], g.wf[1], g.wf[2] };
	float pl[3] = { pa.x, pa.y, pa.z };
#pragma unroll
	for(int a = 0; a < 3; a++) { /* the candidate box (a factor 1 on unscaled axes changes nothing) */
		w[a] *= sf3[a];
		pl[a] *= sf3[a];
	}
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int local = gc - rp.cell_base;
	const int cx = local % nx, cy = (local / nx) % ny, cz = local / (nx * ny);
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float rc2e = rp.sqr_rcut_f + eps;
	const int pslot = __float_as_int(pd.w);
	const float cp[9] = { pb.x, pb.y, pb.z, pb.w, pc.x, pc.y, pc.z, pc.w, pd.x };
	int *partners = (mode == PPI_EN_PARTNERS) ? d.out_partners + (size_t) pslot * PPI_MAX_PARTNERS : nullptr;
	const float4 q0 = make_float4(1.f, 0.f, 0.f, 0.f);
	const float3 d0 = make_float3(0.f, 0.f, 0.f);
	int nb = 0, no = 0;
	for(int t = 0; t < 27 && !(mode == PPI_EN_VOLUME && no); t++) {
		const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
		const int cell = rp.cell_base + (wrapi(cz + dz, nz) * ny + wrapi(cy + dy, ny)) * nx + wrapi(cx + dx, nx);
		const float ox = dx * w[0], oy = dy * w[1], oz = dz * w[2];
		for(int jq = d.cell_start[cell]; jq < d.cell_start[cell + 1]; jq++) {
			if(jq == k) continue;
			const float4 qa = d.spos[jq];
			float ql[3] = { qa.x, qa.y, qa.z };
			ql[0] *= sf3[0];
			ql[1] *= sf3[1];
			ql[2] *= sf3[2];
			const float ddx = (ql[0] - pl[0]) + ox, ddy = (ql[1] - pl[1]) + oy, ddz = (ql[2] - pl[2]) + oz;
			const float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
			A.pairs++;
			if(r2 >= rc2e) continue;
			const float4 qb = d.sori[3 * (size_t) jq], qc = d.sori[3 * (size_t) jq + 1], qd = d.sori[3 * (size_t) jq + 2];
			const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
			const int cl = pair_state<MODE_FAST>(d.rec, rp, rs, g.inv_L, pslot, 0, q0, d0, __float_as_int(qd.w), ddx, ddy, ddz, cp, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps,
					vmask, vf3, vb3, A.fallbacks);
			if(cl == CL_BOND) {
				if(partners && nb < PPI_MAX_PARTNERS) partners[nb] = __float_as_int(qd.y);
				nb++;
			}
			if(cl == CL_OVER) {
				no++;
				if(mode == PPI_EN_VOLUME) break;
			}
		}
	}
	if(mode != PPI_EN_VOLUME) {
		d.out_bonds[pslot] = nb;
		d.out_overlaps[pslot] = no;
	}
	if(no && !rs->vol_overlap) atomicExch(&rs->vol_overlap, 1);
	if(!(mode == PPI_EN_VOLUME && no)) A.tries += nb;
}

/* energy of one particle from scratch, G lanes: bond and overlap counts over all partners (MC_energy,
 * MC.c:272-309, without the early exit, as output_print_bonds counts them, output.c:213-268), or its
 * share of the NPT candidate box's energy (MC.c:487-495). G = 1 in PPI_EN_PARTNERS mode, which also
 * lists the bonded partners. Returns 1 if a pair fell inside the guard band: the particle is then
 * computed again on its own, exactly, at the end of the pass (energy_exact), and nothing is written. */
template <int MODE, int G>
__device__ __forceinline__ int energy_particle(const ppi_dev &d, int mode, int k, Acc &A, const int sub, const unsigned gm) {
	const float4 pa = d.spos[k];
	const float4 pd = d.sori[3 * (size_t) k + 2];
	const int gc = __float_as_int(pd.z);
	const int r = d.cell_rep[gc];
	if(r != A.r) {
		energy_flush_thread(d, A);
		A.r = r;
	}
	const ppi_rparams &rp = d.rp[r];
	const ppi_grid &g = d.grid[r];
	ppi_rstate *rs = d.rs + r;
	int vmask = 0;
	float sf3[3] = { 1.f, 1.f, 1.f };
	const double *vf3 = nullptr, *vb3 = nullptr;
	if(mode == PPI_EN_VOLUME) {
		if(g.vol_dir < 0) return 0;
		/* one overlap already rejects the candidate box: skip (one read per group, shared) */
		int skip = sub == 0 ? *(volatile int *) &rs->vol_overlap : 0;
		skip = __shfl_sync(gm, skip, 0, G);
		if(skip) return 0;
		vmask = g.vol_mask;
		sf3[0] = g.vol_ff3[0];
		sf3[1] = g.vol_ff3[1];
		sf3[2] = g.vol_ff3[2];
		vf3 = g.vol_f3;
		vb3 = g.vol_box3;
	}
	float w[3] = { g.wf[0], g.wf[1], g.wf[2] };
	float pl[3] = { pa.x, pa.y, pa.z };
#pragma unroll
	for(int a = 0; a < 3; a++) { /* the candidate box (a factor 1 on unscaled axes changes nothing) */
		w[a] *= sf3[a];
		pl[a] *= sf3[a];
	}
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int local = gc - rp.cell_base;
	const int cx = local % nx, cy = (local / nx) % ny, cz = local / (nx * ny);
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float sqr_rcut = rp.sqr_rcut_f, cosmax = rp.cosmax_f, basef = rp.base_f, rc2e = sqr_rcut + eps, ovl = 1.f - eps;
	const int pslot = __float_as_int(pd.w);
	int nb = 0, no = 0, uns = 0, u0 = 0, u1 = 0; /* guard-band pairs: count, first two candidates */
	int *partners = (mode == PPI_EN_PARTNERS) ? d.out_partners + (size_t) pslot * PPI_MAX_PARTNERS : nullptr;
	const int *cs = d.cell_start;
	float cp[9];
	{
		const float4 pb = d.sori[3 * (size_t) k], pc = d.sori[3 * (size_t) k + 1];
		cp[0] = pb.x;
		cp[1] = pb.y;
		cp[2] = pb.z;
		cp[3] = pb.w;
		cp[4] = pc.x;
		cp[5] = pc.y;
		cp[6] = pc.z;
		cp[7] = pc.w;
		cp[8] = pd.x;
	}
	const float4 q0 = make_float4(1.f, 0.f, 0.f, 0.f);
	const float3 d0 = make_float3(0.f, 0.f, 0.f);
	const int xm = wrapi(cx - 1, nx), xp = wrapi(cx + 1, nx);
	const int stop_on_overlap = (mode == PPI_EN_VOLUME);
	for(int t = sub; t < 9 && !(stop_on_overlap && no) && uns <= 2; t += G) {
		const int dy = t % 3 - 1, dz = t / 3 - 1;
		const int row = rp.cell_base + (wrapi(cz + dz, nz) * ny + wrapi(cy + dy, ny)) * nx;
		const int a0 = cs[row + xm], a1 = cs[row + xm + 1], m0 = cs[row + cx], m1 = cs[row + cx + 1], p0 = cs[row + xp], p1 = cs[row + xp + 1];
		const float oy = dy * w[1], oz = dz * w[2];
#pragma unroll 1
		for(int c = 0; c < 3 && !(stop_on_overlap && no) && uns <= 2; c++) {
			const float ox = (c - 1) * w[0];
			const int j1 = c == 0 ? a1 : (c == 1 ? m1 : p1);
			for(int jq = (c == 0 ? a0 : (c == 1 ? m0 : p0)); jq < j1; jq++) {
				if(jq == k) continue;
				const float4 qa = d.spos[jq];
				float ql[3] = { qa.x, qa.y, qa.z };
				ql[0] *= sf3[0];
				ql[1] *= sf3[1];
				ql[2] *= sf3[2];
				const float ddx = (ql[0] - pl[0]) + ox, ddy = (ql[1] - pl[1]) + oy, ddz = (ql[2] - pl[2]) + oz;
				const float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
				A.pairs++;
				int cl;
				if(MODE != MODE_AUDIT && r2 < ovl) cl = CL_OVER;
				else if(MODE != MODE_AUDIT && r2 >= rc2e) continue;
				else {
					const float4 qb = d.sori[3 * (size_t) jq], qc = d.sori[3 * (size_t) jq + 1];
					const float4 qd = d.sori[3 * (size_t) jq + 2];
					const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
					if(MODE == MODE_AUDIT)
						cl = pair_state<MODE>(d.rec, rp, rs, g.inv_L, pslot, 0, q0, d0, __float_as_int(qd.w), ddx, ddy, ddz, cp, cq, sqr_rcut, cosmax, basef, eps, vmask, vf3, vb3, A.fallbacks);
					else {
						cl = classify(ddx, ddy, ddz, cp, cq, sqr_rcut, cosmax, basef, eps, nullptr);
						if(cl == CL_UNSURE) { /* decided after the loop by the certified FP64 test */
							if(uns == 0) u0 = jq;
							else u1 = jq;
							if(++uns > 2) break;
							continue;
						}
					}
					if(cl == CL_BOND && partners && nb < PPI_MAX_PARTNERS) partners[nb] = __float_as_int(qd.y);
				}
				nb += (cl == CL_BOND);
				if(cl == CL_OVER) {
					no++;
					if(stop_on_overlap) break;
				}
			}
		}
	}
	if(MODE == MODE_FAST && uns && !(stop_on_overlap && no)) {
		if(uns > 2) uns = -1; /* more than this lane keeps: the particle is computed exactly at the end */
		else
			for(int k2 = 0; k2 < uns; k2++) {
				const int jq = k2 ? u1 : u0;
				const float4 qd = d.sori[3 * (size_t) jq + 2];
				A.fallbacks++;
				const int ex = decide64(d.rec, rp, rs->box, g.inv_L, pslot, 0, q0, d0, __float_as_int(qd.w), vmask, vf3, vb3);
				if(ex == DEC64_EXACT) {
					uns = -1;
					break;
				}
				if(ex == 1) {
					if(partners && nb < PPI_MAX_PARTNERS) partners[nb] = __float_as_int(qd.y);
					nb++;
				}
				no += (ex == -1);
			}
	}
	if(MODE == MODE_FAST && __any_sync(gm, uns < 0)) return 1;
	nb = group_sum<G>(gm, nb);
	no = group_sum<G>(gm, no);
	if(sub == 0) {
		if(mode != PPI_EN_VOLUME) {
			d.out_bonds[pslot] = nb;
			d.out_overlaps[pslot] = no;
		}
		if(no && !rs->vol_overlap) atomicExch(&rs->vol_overlap, 1); /* visible at once: lets the others skip work */
		if(!(mode == PPI_EN_VOLUME && no)) A.tries += nb;
	}
	return 0;
}

#define ENERGY_DCAP 16 /* deferred particles a warp keeps in shared memory (more: flags in global memory) */

template <int MODE, int G>
__global__ void __launch_bounds__(128, MODE == MODE_FAST ? PPI_FAST_MIN_BLOCKS : 1) k_energy(ppi_dev d, int mode) {
	__shared__ int s_dl[4][ENERGY_DCAP];
	__shared__ int s_nd[4], s_dov[4];
	constexpr int PW = 32 / G;
	if(blockIdx.x * (blockDim.x / G) >= d.ntot) return;
	Acc A; /* A.tries = bonds counted, pairs, fallbacks */
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
	const int sub = threadIdx.x & (G - 1), slot = (threadIdx.x & 31) / G;
	const unsigned gm = group_mask<G>();
	if(lane == 0) {
		s_nd[wi] = 0;
		s_dov[wi] = 0;
	}
	__syncwarp();
	for(int b = warp * PW; b < d.ntot; b += nwarp * PW) {
		const int k = b + slot;
		if(k < d.ntot && energy_particle<MODE, G>(d, mode, k, A, sub, gm) && sub == 0) {
			const int i = atomicAdd(&s_nd[wi], 1);
			if(i < ENERGY_DCAP) s_dl[wi][i] = k;
			else {
				d.eflag[k] = 1;
				s_dov[wi] = 1;
			}
		}
	}
	__syncwarp();
	/* the deferred particles, one per lane, exactly */
	const int nd = s_nd[wi] < ENERGY_DCAP ? s_nd[wi] : ENERGY_DCAP;
	for(int i = lane; i < nd; i += 32) energy_exact(d, mode, s_dl[wi][i], A);
	if(s_dov[wi])
		for(int b = warp * PW; b < d.ntot; b += nwarp * PW)
			if(sub == 0 && b + slot < d.ntot && d.eflag[b + slot]) {
				d.eflag[b + slot] = 0;
				energy_exact(d, mode, b + slot, A);
			}
	__syncwarp();
	energy_flush_block(d, A);
}

/* ------------------------------------------------------------------------------------------------ */
/* NPT candidate box: bonds and overlaps of all pairs, one warp tile of 64 particles at a time       */
/* ------------------------------------------------------------------------------------------------ */
/* The volume move needs only the candidate box's total bond count and whether any pair overlaps
 * (MC.c:487-495), so every pair is evaluated once, from its particle with the lower sorted position
 * (a half shell: each row range of the neighbourhood is clamped to positions above the particle's).
 * Same pair-list layout as the colour pass: lanes own particles for the set-up, the pairs of a plane are
 * flattened and walked 32 per step, pairs within the bonding range get their patch test, guard-band pairs
 * the certified FP64 test and, in the rare undecided case, exact_pair at the end of the warp's share. */
#define EV_UCAP 32

struct __align__(16) VolSmem {
	float4 pos[TA];   /* scaled cell-local position, .w = cell x index */
	float4 wv[TA];    /* scaled cell edges, .w = number of x cells */
	float4 vs[TA];    /* (-, -, 1 - eps, r_cut^2 + eps) */
	float4 sc[TA];    /* scale factors of the candidate box per axis (1 on unscaled axes) */
	float cp[9][TA];  /* orientation columns */
	int ki[TA];       /* sorted position */
	int rep[TA];
	int cc[TA];       /* cell coordinates cx | cy << 10 | cz << 20, -1: no particle */
	int pbuf[TILE_PCAP]; /* (candidate - particle) << 10 | particle << 4 | row */
	int cbuf[TILE_CCAP];
	int2 uns[EV_UCAP];  /* guard-band pairs: (candidate, particle) */
	int2 exl[EV_UCAP];  /* pairs left to exact_pair: (candidate, particle), decided at the end of the share */
	int nc, nu, nex;
};

__device__ __forceinline__ void vol_exact_later(const ppi_dev &d, VolSmem &S, int jq, int k);

__device__ __forceinline__ void vol_setup(const ppi_dev &d, VolSmem &S, int a, int k) {
	int cc = -1, r = 0;
	float4 pos = make_float4(0.f, 0.f, 0.f, 0.f), wv = make_float4(1.f, 1.f, 1.f, __int_as_float(4)), vs = make_float4(0.f, 0.f, 0.f, 0.f);
	float4 sc = make_float4(1.f, 1.f, 1.f, 0.f);
	if(k >= 0) {
		const float4 pa = d.spos[k], pb = d.sori[3 * (size_t) k], pc = d.sori[3 * (size_t) k + 1], pd = d.sori[3 * (size_t) k + 2];
		const int gc = __float_as_int(pd.z);
		r = d.cell_rep[gc];
		const ppi_grid &g = d.grid[r];
		if(g.vol_dir >= 0) {
			sc = make_float4(g.vol_ff3[0], g.vol_ff3[1], g.vol_ff3[2], 0.f);
			pos = make_float4(pa.x * sc.x, pa.y * sc.y, pa.z * sc.z, pa.w);
			wv = make_float4(g.wf[0] * sc.x, g.wf[1] * sc.y, g.wf[2] * sc.z, __int_as_float(g.n[0]));
			const ppi_rparams &rp = d.rp[r];
			const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
			vs = make_float4(0.f, 0.f, 1.f - eps, rp.sqr_rcut_f + eps);
			const int local = gc - d.rp[r].cell_base;
			cc = (local % g.n[0]) | (((local / g.n[0]) % g.n[1]) << 10) | ((local / (g.n[0] * g.n[1])) << 20);
			const float c9[9] = { pb.x, pb.y, pb.z, pb.w, pc.x, pc.y, pc.z, pc.w, pd.x };
#pragma unroll
			for(int j = 0; j < 9; j++) S.cp[j][a] = c9[j];
		}
	}
	S.pos[a] = pos;
	S.wv[a] = wv;
	S.vs[a] = vs;
	S.sc[a] = sc;
	S.ki[a] = k;
	S.rep[a] = r;
	S.cc[a] = cc;
}

/* half-shell ranges of plane pz of particle a (candidates above its sorted position) */
__device__ __forceinline__ int vol_ranges(const ppi_dev &d, const VolSmem &S, int a, int pz, PlaneRanges &P) {
#pragma unroll
	for(int j = 0; j < 6; j++) P.s[j] = P.e[j] = 0;
	const int ccp = S.cc[a];
	if(ccp < 0) return 0;
	const int r = S.rep[a];
	if(*(volatile int *) &d.rs[r].vol_overlap) return 0; /* the candidate box is rejected already */
	const ppi_grid &g = d.grid[r];
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int cb = d.rp[r].cell_base;
	const int cx = ccp & 1023, cy = (ccp >> 10) & 1023, cz = ccp >> 20;
	const bool inner = cx >= 1 && cx <= nx - 2;
	const int xa0 = inner ? cx - 1 : (cx == 0 ? nx - 1 : nx - 2), xa1 = inner ? cx + 2 : nx;
	const int xb1 = cx == 0 ? 2 : 1;
	const int kmin = S.ki[a] + 1;
	int n = 0;
#pragma unroll
	for(int ry = 0; ry < 3; ry++) {
		const int *cs = d.cell_start + cb + (wrapi(cz + pz - 1, nz) * ny + wrapi(cy + ry - 1, ny)) * nx;
		P.s[2 * ry] = max(cs[xa0], kmin);
		P.e[2 * ry] = max(cs[xa1], P.s[2 * ry]);
		if(!inner) {
			P.s[2 * ry + 1] = max(cs[0], kmin);
			P.e[2 * ry + 1] = max(cs[xb1], P.s[2 * ry + 1]);
		}
	}
#pragma unroll
	for(int j = 0; j < 6; j++) n += P.e[j] - P.s[j];
	return n;
}

__device__ __forceinline__ int vol_far(const VolSmem &S, int a, const PlaneRanges &P) {
	int m = 0;
#pragma unroll
	for(int j = 0; j < 6; j++) m = max(m, P.e[j]);
	return m - S.ki[a] >= TILE_OFF_MAX;
}

__device__ __forceinline__ void vol_write(VolSmem &S, int a, int pz, const PlaneRanges &P, int pos) {
	const int k = S.ki[a];
#pragma unroll
	for(int sg = 0; sg < 6; sg++) {
		const int tag = (a << 4) | (3 * pz + (sg >> 1));
		for(int jq = P.s[sg]; jq < P.e[sg]; jq++) {
			const int off = jq - k;
			S.pbuf[pos++] = (int) ((unsigned) off << 10) | tag;
		}
	}
}

/* candidate position in particle a's scaled cell frame, relative to a */
__device__ __forceinline__ float3 vol_geo(const VolSmem &S, int a, int t, float4 qa) {
	const float4 p = S.pos[a], w = S.wv[a], c = S.sc[a];
	const float qx = qa.x * c.x, qy = qa.y * c.y, qz = qa.z * c.z;
	const int nxc = __float_as_int(w.w);
	int dxc = __float_as_int(qa.w) - __float_as_int(p.w);
	dxc = dxc > 1 ? dxc - nxc : (dxc < -1 ? dxc + nxc : dxc);
	return make_float3((qx - p.x) + dxc * w.x, (qy - p.y) + (t % 3 - 1) * w.y, (qz - p.z) + (t / 3 - 1) * w.z);
}

__device__ __forceinline__ void vol_close(const ppi_dev &d, VolSmem &S, int lane, Acc &A) {
	const int nc = S.nc;
	for(int c = lane; c < nc; c += 32) {
		const int en = S.cbuf[c];
		const int a = (en >> 4) & 63, t = en & 15;
		const int jq = S.ki[a] + (en >> 10);
		const int r = S.rep[a];
		const ppi_rparams &rp = d.rp[r];
		const float4 qa = d.spos[jq], qb = d.sori[3 * (size_t) jq], qc = d.sori[3 * (size_t) jq + 1], qd = d.sori[3 * (size_t) jq + 2];
		const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd.x };
		float cp[9];
#pragma unroll
		for(int j = 0; j < 9; j++) cp[j] = S.cp[j][a];
		const float3 dv = vol_geo(S, a, t, qa);
		const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
		const int cl = classify(dv.x, dv.y, dv.z, cp, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, nullptr);
		if(cl == CL_UNSURE) {
			const int k = atomicAdd(&S.nu, 1);
			if(k < EV_UCAP) S.uns[k] = make_int2(jq, a);
			else vol_exact_later(d, S, jq, S.ki[a]); /* list full: decided exactly at the end */
			continue;
		}
		if(r != A.r) {
			energy_flush_thread(d, A);
			A.r = r;
		}
		if(cl == CL_BOND) A.tries += 2; /* the box total counts every bond from both sides */
		else if(cl == CL_OVER && !d.rs[r].vol_overlap) atomicExch(&d.rs[r].vol_overlap, 1);
	}
	__syncwarp();
	if(lane == 0) S.nc = 0;
	__syncwarp();
}

/* a pair for exact_pair at the end of the warp's share; more than EV_UCAP of them in one share (pairs
 * within 1e-12 of a threshold, or guard-band overflow) is reported as PPI_E_EXACT instead */
__device__ __forceinline__ void vol_exact_later(const ppi_dev &d, VolSmem &S, int jq, int k) {
	const int x = atomicAdd(&S.nex, 1);
	if(x < EV_UCAP) S.exl[x] = make_int2(jq, k);
	else d.rs[d.cell_rep[__float_as_int(d.sori[3 * (size_t) k + 2].z)]].error = PPI_E_EXACT;
}

/* the decision of pair (candidate jq, particle k): certified FP64 (in the loop), or the bit-identical
 * exact_pair (after the loop, for the pairs the certified test leaves undecided) */
template <bool EXACT>
__device__ __forceinline__ void vol_pair_decide(const ppi_dev &d, VolSmem &S, int jq, int k, Acc &A) {
	const int r = d.cell_rep[__float_as_int(d.sori[3 * (size_t) k + 2].z)];
	const ppi_grid &g = d.grid[r];
	const int ps = __float_as_int(d.sori[3 * (size_t) k + 2].w), qs = __float_as_int(d.sori[3 * (size_t) jq + 2].w);
	const float4 q0 = make_float4(1.f, 0.f, 0.f, 0.f);
	const float3 d0 = make_float3(0.f, 0.f, 0.f);
	A.fallbacks++;
	int ex;
	if(EXACT) ex = exact_pair(d.rec, d.rp + r, d.rs[r].box, ps, 0, q0, d0, qs, g.vol_mask, g.vol_f3, g.vol_box3, nullptr, nullptr, nullptr);
	else {
		ex = decide64(d.rec, d.rp[r], d.rs[r].box, g.inv_L, ps, 0, q0, d0, qs, g.vol_mask, g.vol_f3, g.vol_box3);
		if(ex == DEC64_EXACT) {
			vol_exact_later(d, S, jq, k);
			return;
		}
	}
	if(r != A.r) {
		energy_flush_thread(d, A);
		A.r = r;
	}
	if(ex == 1) A.tries += 2; /* the box total counts every bond from both sides */
	else if(ex == -1 && !d.rs[r].vol_overlap) atomicExch(&d.rs[r].vol_overlap, 1);
}

/* the pairs of a lane whose plane slice alone exceeds the pair list (cells far denser than a hard-sphere
 * packing allows; kept for completeness): evaluated one by one */
__device__ __forceinline__ void vol_lane_pairs(const ppi_dev &d, VolSmem &S, int a, int pz, const PlaneRanges &P, Acc &A) {
	const int k = S.ki[a];
	const int r = S.rep[a];
	const ppi_rparams &rp = d.rp[r];
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	float cp[9];
#pragma unroll
	for(int j = 0; j < 9; j++) cp[j] = S.cp[j][a];
	for(int sg = 0; sg < 6; sg++)
		for(int jq = P.s[sg]; jq < P.e[sg]; jq++) {
			const float4 qa = d.spos[jq], qb = d.sori[3 * (size_t) jq], qc = d.sori[3 * (size_t) jq + 1];
			const float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, d.sori[3 * (size_t) jq + 2].x };
			const float3 dv = vol_geo(S, a, 3 * pz + (sg >> 1), qa);
			A.pairs++;
			const int cl = classify(dv.x, dv.y, dv.z, cp, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, eps, nullptr);
			if(cl == CL_UNSURE) vol_pair_decide<false>(d, S, jq, k, A);
			else {
				if(r != A.r) {
					energy_flush_thread(d, A);
					A.r = r;
				}
				if(cl == CL_BOND) A.tries += 2;
				else if(cl == CL_OVER && !d.rs[r].vol_overlap) atomicExch(&d.rs[r].vol_overlap, 1);
			}
		}
}

/* the pair list's np entries, PSTEP steps of 32 pairs at a time: certain overlaps, close pairs compacted
 * into the patch-test list */
__device__ __forceinline__ void vol_steps(const ppi_dev &d, VolSmem &S, const int lane, const int np, Acc &A) {
	const unsigned lt = (1u << lane) - 1u;
	for(int p0 = 0; p0 < np; p0 += 32 * PSTEP) {
		int en[PSTEP], ok[PSTEP];
		float4 qa[PSTEP];
#pragma unroll
		for(int u = 0; u < PSTEP; u++) {
			const int p = p0 + 32 * u + lane;
			en[u] = 0;
			ok[u] = 0;
			qa[u] = make_float4(0.f, 0.f, 0.f, 0.f);
			if(p < np) {
				en[u] = S.pbuf[p];
				const int a = (en[u] >> 4) & 63, off = en[u] >> 10;
				ok[u] = off != 0;
				if(ok[u]) qa[u] = d.spos[S.ki[a] + off];
			}
		}
#pragma unroll
		for(int u = 0; u < PSTEP; u++) {
			int close = 0;
			if(ok[u]) {
				const int a = (en[u] >> 4) & 63;
				const float3 dv = vol_geo(S, a, en[u] & 15, qa[u]);
				const float r2 = fmaf(dv.x, dv.x, fmaf(dv.y, dv.y, dv.z * dv.z));
				const float4 v = S.vs[a];
				A.pairs++;
				if(r2 < v.z) {
					const int r = S.rep[a];
					if(!d.rs[r].vol_overlap) atomicExch(&d.rs[r].vol_overlap, 1);
				}
				else close = r2 < v.w;
			}
			const unsigned m = __ballot_sync(0xffffffffu, close);
			if(m) {
				if(S.nc + __popc(m) > TILE_CCAP) vol_close(d, S, lane, A);
				if(close) S.cbuf[S.nc + __popc(m & lt)] = en[u];
				__syncwarp();
				if(lane == 0) S.nc += __popc(m);
				__syncwarp();
			}
		}
	}
}

/* particle a's pairs from its neighbour list, each pair once (from the lower sorted position): the number
 * of entries above a's position; far = 1 when a's list overflowed or holds a candidate farther than a
 * packed entry reaches (a's half shell is then evaluated one by one) */
__device__ __forceinline__ int vol_list_count(const ppi_dev &d, const VolSmem &S, int a, int &far) {
	far = 0;
	const int k = S.ki[a];
	if(S.cc[a] < 0 || *(volatile int *) &d.rs[S.rep[a]].vol_overlap) return 0;
	const int n = d.nl_cnt[k];
	if(n > d.nl_k) {
		far = 1;
		return 0;
	}
	const int4 *L = (const int4 *) (d.nl + (size_t) k * d.nl_k);
	int c = 0;
	for(int k0 = 0; k0 < n; k0 += 4) {
		const int4 v = L[k0 >> 2];
		const int e4[4] = { v.x, v.y, v.z, v.w };
#pragma unroll
		for(int u = 0; u < 4; u++) {
			const int jq = (int) ((unsigned) e4[u] >> 5);
			if(k0 + u < n && jq > k) {
				c++;
				far |= jq - k >= TILE_OFF_MAX;
			}
		}
	}
	return far ? 0 : c;
}

/* the entries counted by vol_list_count into the pair list from position pos (row tag = code / 3) */
__device__ __forceinline__ void vol_list_write(const ppi_dev &d, VolSmem &S, int a, int pos) {
	const int k = S.ki[a];
	const int n = d.nl_cnt[k];
	const int4 *L = (const int4 *) (d.nl + (size_t) k * d.nl_k);
	for(int k0 = 0; k0 < n; k0 += 4) {
		const int4 v = L[k0 >> 2];
		const int e4[4] = { v.x, v.y, v.z, v.w };
#pragma unroll
		for(int u = 0; u < 4; u++) {
			const int jq = (int) ((unsigned) e4[u] >> 5);
			if(k0 + u < n && jq > k) S.pbuf[pos++] = (int) ((unsigned) (jq - k) << 10) | (a << 4) | ((e4[u] & 31) / 3);
		}
	}
}

template <bool LIST>
__global__ void __launch_bounds__(32 * TILE_WARPS, PPI_VOL_MIN_BLOCKS) k_energy_vol(ppi_dev d) {
	__shared__ VolSmem s_vol[TILE_WARPS];
	VolSmem &S = s_vol[threadIdx.x >> 5];
	const int lane = threadIdx.x & 31;
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
	const int lo = (int) ((long long) warp * d.ntot / nwarp), hi = (int) ((long long) (warp + 1) * d.ntot / nwarp);
	if(lane == 0) S.nex = 0;
	__syncwarp();
	for(int b = lo; b < hi; b += TA) {
		vol_setup(d, S, lane, b + lane < hi ? b + lane : -1);
		vol_setup(d, S, lane + 32, b + 32 + lane < hi ? b + 32 + lane : -1);
		if(lane == 0) {
			S.nc = 0;
			S.nu = 0;
		}
		__syncwarp();
		if(LIST) { /* pairs from the neighbour lists, one half of the particles (a lane each) at a time */
#pragma unroll 1
			for(int h = 0; h < 2; h++) {
				const int a = lane + 32 * h;
				int far;
				const int n = vol_list_count(d, S, a, far);
				if(far) {
#pragma unroll 1
					for(int pz = 0; pz < 3; pz++) {
						PlaneRanges P;
						vol_ranges(d, S, a, pz, P);
						vol_lane_pairs(d, S, a, pz, P, A);
					}
				}
				int incl = n;
#pragma unroll
				for(int o = 1; o < 32; o <<= 1) {
					const int v = __shfl_up_sync(0xffffffffu, incl, o);
					if(lane >= o) incl += v;
				}
				const int total = __shfl_sync(0xffffffffu, incl, 31);
				int done = 0;
				while(done < total) { /* lanes whose slices fit together (a slice is at most nl_k <= TILE_PCAP) */
					const int start = incl - n;
					const int mine = n > 0 && start >= done && incl - done <= TILE_PCAP;
					const unsigned take = __ballot_sync(0xffffffffu, mine);
					if(take == 0) break; /* unreachable while nl_k <= TILE_PCAP */
					if(mine) vol_list_write(d, S, a, start - done);
					const int end = __shfl_sync(0xffffffffu, incl, 31 - __clz(take));
					__syncwarp();
					vol_steps(d, S, lane, end - done, A);
					done = end;
					__syncwarp();
				}
			}
		}
#pragma unroll 1
		for(int pz = 0; pz < (LIST ? 0 : 3); pz++) {
			PlaneRanges P0, P1;
			int n0 = vol_ranges(d, S, lane, pz, P0), n1 = vol_ranges(d, S, lane + 32, pz, P1);
			/* candidates farther than a packed entry can hold (planes of more than ~2M particles): one by one */
			if(n0 && vol_far(S, lane, P0)) {
				vol_lane_pairs(d, S, lane, pz, P0, A);
				n0 = 0;
#pragma unroll
				for(int j = 0; j < 6; j++) P0.s[j] = P0.e[j] = 0;
			}
			if(n1 && vol_far(S, lane + 32, P1)) {
				vol_lane_pairs(d, S, lane + 32, pz, P1, A);
				n1 = 0;
#pragma unroll
				for(int j = 0; j < 6; j++) P1.s[j] = P1.e[j] = 0;
			}
			const int n = n0 + n1;
			int incl = n;
#pragma unroll
			for(int o = 1; o < 32; o <<= 1) {
				const int v = __shfl_up_sync(0xffffffffu, incl, o);
				if(lane >= o) incl += v;
			}
			const int total = __shfl_sync(0xffffffffu, incl, 31);
			if(total == 0) continue;
			/* a plane that does not fit is walked in slices of whole lanes */
			int done = 0;
			while(done < total) {
				const int start = incl - n;
				const int mine = n > 0 && start >= done && incl - done <= TILE_PCAP;
				const unsigned take = __ballot_sync(0xffffffffu, mine);
				if(take == 0) { /* the next lane's slice alone exceeds the list */
					const int big = n > 0 && start == done;
					if(big) {
						vol_lane_pairs(d, S, lane, pz, P0, A);
						vol_lane_pairs(d, S, lane + 32, pz, P1, A);
					}
					const unsigned bm = __ballot_sync(0xffffffffu, big);
					done = __shfl_sync(0xffffffffu, incl, __ffs(bm) - 1);
					continue;
				}
				if(mine) {
					const int pos = start - done;
					vol_write(S, lane, pz, P0, pos);
					vol_write(S, lane + 32, pz, P1, pos + n0);
				}
				const int end = __shfl_sync(0xffffffffu, incl, 31 - __clz(take));
				const int np = end - done;
				__syncwarp();
				vol_steps(d, S, lane, np, A);
				done = end;
				__syncwarp();
			}
		}
		if(S.nc) vol_close(d, S, lane, A);
		/* guard-band pairs: certified FP64 decisions */
		const int nu = S.nu < EV_UCAP ? S.nu : EV_UCAP;
		for(int u = lane; u < nu; u += 32) vol_pair_decide<false>(d, S, S.uns[u].x, S.ki[S.uns[u].y], A);
		__syncwarp();
	}
	/* pairs within 1e-12 of a threshold (rare): the bit-identical exact_pair, after the loop */
	const int nex = S.nex < EV_UCAP ? S.nex : EV_UCAP;
	for(int u = lane; u < nex; u += 32) vol_pair_decide<true>(d, S, S.exl[u].x, S.exl[u].y, A);
	__syncwarp();
	energy_flush_block(d, A);
}

/* the candidate box of one replica as the flat volume pass uses it (kept in registers across pairs) */
struct VolRep {
	int r, live;       /* replica; live: it has a candidate box this sweep and no overlap was found yet */
	float sx, sy, sz;  /* scale factors per axis */
	float wx, wy, wz;  /* scaled cell edges */
	float ovl, rc2e;   /* 1 - eps, r_cut^2 + eps */
	float eps;
};

__device__ __forceinline__ void vol_rep_load(const ppi_dev &d, int r, VolRep &V) {
	const ppi_grid &g = d.grid[r];
	const ppi_rparams &rp = d.rp[r];
	V.r = r;
	V.live = g.vol_dir >= 0 && !*(volatile int *) &d.rs[r].vol_overlap;
	V.sx = g.vol_ff3[0];
	V.sy = g.vol_ff3[1];
	V.sz = g.vol_ff3[2];
	V.wx = g.wf[0] * V.sx;
	V.wy = g.wf[1] * V.sy;
	V.wz = g.wf[2] * V.sz;
	V.eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	V.ovl = 1.f - V.eps;
	V.rc2e = rp.sqr_rcut_f + V.eps;
}

/* one pair (lower sorted position i, candidate jq, cell offset code) of the candidate box, the positions
 * already loaded; the geometry is vol_geo's */
__device__ __forceinline__ void vol_flat_pair(const ppi_dev &d, const VolRep &V, const int i, const int jq, const int code, const float4 pa, const float4 qa,
		Acc &A) {
	const float ex = (qa.x * V.sx - pa.x * V.sx) + (float) (code % 3 - 1) * V.wx;
	const float ey = (qa.y * V.sy - pa.y * V.sy) + (float) ((code / 3) % 3 - 1) * V.wy;
	const float ez = (qa.z * V.sz - pa.z * V.sz) + (float) (code / 9 - 1) * V.wz;
	const float r2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
	ppi_rstate *rs = d.rs + V.r;
	A.pairs++;
	if(r2 < V.ovl) {
		atomicExch(&rs->vol_overlap, 1);
		return;
	}
	if(!(r2 < V.rc2e)) return;
	const ppi_rparams &rp = d.rp[V.r];
	const float4 p0 = d.sori[3 * (size_t) i], p1 = d.sori[3 * (size_t) i + 1], p2 = d.sori[3 * (size_t) i + 2];
	const float4 q0 = d.sori[3 * (size_t) jq], q1 = d.sori[3 * (size_t) jq + 1], q2 = d.sori[3 * (size_t) jq + 2];
	const float cp[9] = { p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w, p2.x };
	const float cq[9] = { q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x };
	int pv;
	const int cl = classify_pv(ex, ey, ez, cp, cq, rp.sqr_rcut_f, rp.cosmax_f, rp.base_f, V.eps, &pv);
	if(cl == CL_UNSURE) { /* guard band: queued for the FP64 decision after the pass (k_vol_unsure), with its patch verdict */
		const int k = atomicAdd(d.vun_count, 1);
		if(k < d.vun_cap) d.vunsure[k] = make_int2(i, jq | (pv << 28)); /* sorted positions are below 2^27 */
		else rs->error = PPI_E_LISTS;
	}
	else if(cl == CL_BOND) A.tries += 2; /* the box total counts every bond from both sides */
	else if(cl == CL_OVER) atomicExch(&rs->vol_overlap, 1);
}

/* Energy of the candidate box of the sweep (NPT volume move or Lx move) over the epoch's flat pair list:
 * one thread per pair (lower sorted position i, candidate jq), the positions and cell edges scaled axis by
 * axis as in vol_geo; bonds counted from both sides (rs.vol_bonds = 2 x bonds), any overlap flags the
 * replica. The list holds every pair that can interact in any candidate box of the epoch. A thread loads
 * its next pair while it evaluates the current one, and keeps its replica's candidate box in registers
 * (the overlap flag is re-read every few steps: a rejected box only saves work). */
#define VP_B 128
#ifndef PPI_VP_MIN_BLOCKS
#define PPI_VP_MIN_BLOCKS 8 /* resident CTAs per SM of the flat volume pass (64 registers) */
#endif
__global__ void __launch_bounds__(VP_B, PPI_VP_MIN_BLOCKS) k_energy_vol_pairs(ppi_dev d) {
	grid_dep_wait();
	grid_dep_release();
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	VolRep V;
	V.r = -1;
	V.live = 0;
	const int np = d.vp_count[0] < d.vp_cap ? d.vp_count[0] : d.vp_cap;
	const int nth = gridDim.x * blockDim.x, first = blockIdx.x * blockDim.x + threadIdx.x;
	/* software pipeline: the next pair's loads are in flight while the current pair is evaluated */
	int p = first, step = 0;
	int2 c = p < np ? d.vpairs[p] : make_int2(-1, 0);
	int rc = 0;
	float4 pc = make_float4(0.f, 0.f, 0.f, 0.f), qc = pc;
	if(c.x >= 0) {
		rc = d.srep[c.x];
		pc = d.spos[c.x];
		qc = d.spos[(unsigned) c.y >> 5];
	}
	while(c.x >= 0) {
		const int pn = p + nth;
		int2 n = pn < np ? d.vpairs[pn] : make_int2(-1, 0);
		int rn = 0;
		float4 pnx = pc, qnx = qc;
		if(n.x >= 0) {
			rn = d.srep[n.x];
			pnx = d.spos[n.x];
			qnx = d.spos[(unsigned) n.y >> 5];
		}
		if(rc != V.r || (step & 15) == 0) vol_rep_load(d, rc, V);
		if(rc != A.r) {
			energy_flush_thread(d, A);
			A.r = rc;
		}
		if(V.live) vol_flat_pair(d, V, c.x, (int) ((unsigned) c.y >> 5), c.y & 31, pc, qc, A);
		c = n;
		rc = rn;
		pc = pnx;
		qc = qnx;
		p = pn;
		step++;
	}
	/* particles whose list overflowed: their half shell in the 27 cells, one candidate at a time */
	const int no = d.vp_count[1];
	for(int k = first; k < no; k += nth) {
		const int i = d.vp_over[k];
		const int gc = __float_as_int(d.sori[3 * (size_t) i + 2].z);
		const int r = d.cell_rep[gc];
		const ppi_rparams &rp = d.rp[r];
		const ppi_grid &g = d.grid[r];
		vol_rep_load(d, r, V);
		if(!V.live) continue;
		if(r != A.r) {
			energy_flush_thread(d, A);
			A.r = r;
		}
		const int nx = g.n[0], local = gc - rp.cell_base;
		const int cx = local % nx;
		const float4 pa = d.spos[i];
		nl_rows(d, i, rp, g, cx, (local / nx) % g.n[1], local / (nx * g.n[1]), [&](int jq, int dy, int dz) {
			if(jq <= i) return;
			const float4 qa = d.spos[jq];
			int dxc = __float_as_int(qa.w) - cx;
			dxc = dxc > 1 ? dxc - nx : (dxc < -1 ? dxc + nx : dxc);
			vol_flat_pair(d, V, i, jq, (dxc + 1) + 3 * (dy + 1) + 9 * (dz + 1), pa, qa, A);
		});
	}
	energy_flush_block(d, A);
}

/* the guard-band pairs of the flat volume pass: the certified FP64 decision, the bit-identical exact_pair
 * where it cannot decide */
__global__ void k_vol_unsure(ppi_dev d) {
	grid_dep_wait();
	grid_dep_release();
	const int n = d.vun_count[0] < d.vun_cap ? d.vun_count[0] : d.vun_cap;
	/* one warp per pair (decide64_warp); the bit-identical exact test for the rare undecided one */
	const int lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
	const float4 q0 = make_float4(1.f, 0.f, 0.f, 0.f);
	const float3 d0 = make_float3(0.f, 0.f, 0.f);
	for(int k = warp; k < n; k += nwarp) {
		const int2 pr = d.vunsure[k];
		const int jq = pr.y & ((1 << 28) - 1), pv = (unsigned) pr.y >> 28;
		const int r = d.srep[pr.x];
		ppi_rstate *rs = d.rs + r;
		const ppi_grid *g = d.grid + r;
		const int ps = __float_as_int(d.sori[3 * (size_t) pr.x + 2].w), qs = __float_as_int(d.sori[3 * (size_t) jq + 2].w);
		int x = decide64_warp(d.rec, d.rp[r], rs->box, g->inv_L, ps, 0, q0, d0, qs, g->vol_mask, g->vol_f3, g->vol_box3, lane, pv);
		if(lane == 0) {
			if(x == DEC64_EXACT) x = exact_pair(d.rec, d.rp + r, rs->box, ps, 0, q0, d0, qs, g->vol_mask, g->vol_f3, g->vol_box3, nullptr, nullptr, nullptr);
			atomicAdd(&rs->fallbacks, 1ull);
			if(x == 1) atomicAdd((unsigned long long *) &rs->vol_bonds, 2ull);
			else if(x == -1) atomicExch(&rs->vol_overlap, 1);
		}
	}
}

__global__ void k_energy_reset(ppi_dev d) {
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	d.rs[r].vol_bonds = 0;
	d.rs[r].vol_overlap = 0;
	d.rs[r].vol_accept = 0;
}

/* ------------------------------------------------------------------------------------------------ */
/* NPT volume move (MC.c:450-513) and NVT box-shape move (MC.c:515-585)                             */
/* ------------------------------------------------------------------------------------------------ */
/* the candidate box of the sweep: an NPT volume move (MC.c:456-472) or, for NVT replicas with Lx_move, a
 * box-shape move (MC_change_Lx, MC.c:520-537): Lx changes by (R - 0.5) Lx_change_max, Ly = Lz =
 * sqrt(V / Lx) keep the volume, every coordinate is rescaled by its side's factor */
__global__ void k_vol_plan(ppi_dev d, long long sweep) {
	grid_dep_wait(); /* the volume move's kernels are chained by programmatic dependent launch */
	grid_dep_release();
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	sweep = ctr_index(sweep, sweep < 0 ? d.ctr->sweep : 0);
	if(r == 0) {
		d.ctr->vol_any = 0;
		if(d.vun_count) d.vun_count[0] = 0;
	}
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	ppi_grid *g = d.grid + r;
	rs->vol_bonds = 0;
	rs->vol_overlap = 0;
	rs->vol_accept = 0;
	g->vol_dir = -1;
	g->vol_mask = 0;
	for(int k = 0; k < 3; k++) {
		g->vol_f3[k] = 1.0;
		g->vol_box3[k] = rs->box[k];
		g->vol_ff3[k] = 1.f;
	}
	if(rp.N <= 0) return;
	U4 u = rng(rp, sweep, r, TAG_VOL, 0, 0);
	if(rp.ensemble == 5) {
		/* random axis, ln V' = ln V + (R - 0.5) rescale_factor_max, one side takes the whole change */
		int dir = (int) (u01d(u.x, u.y) * 3.0);
		if(dir > 2) dir = 2;
		double V0 = rs->box[0] * rs->box[1] * rs->box[2];
		double lnV = log(V0) + (u01d(u.z, u.w) - 0.5) * rp.rescale_max;
		double V1 = exp(lnV);
		double side = V1;
		for(int i = 0; i < 3; i++)
			if(i != dir) side /= rs->box[i];
		g->vol_dir = dir;
		g->vol_mask = 1 << dir;
		g->vol_f = side / rs->box[dir];
		g->vol_f3[dir] = g->vol_f;
		g->vol_box3[dir] = side;
		g->vol_ff3[dir] = (float) g->vol_f;
		g->vol_V0 = V0;
		g->vol_V1 = V1;
		return;
	}
	if(!rp.lx_move) return;
	const double lx = rs->box[0] + (u01d(u.x, u.y) - 0.5) * rp.lx_change_max;
	const double lyz = sqrt(rs->V / lx);
	/* early rejection (MC.c:526-530); a non-positive Lx (Lx_change_max above twice the side) is rejected too */
	if(!(lx > 0.) || lyz < rp.lyz_min || lyz > rp.lyz_max) {
		rs->tries[7]++;
		return;
	}
	const double nb[3] = { lx, lyz, lyz };
	for(int k = 0; k < 3; k++) {
		g->vol_box3[k] = nb[k];
		g->vol_f3[k] = nb[k] / rs->box[k]; /* rescale_factors (MC.c:533-537) */
		g->vol_ff3[k] = (float) g->vol_f3[k];
		if(g->w[k] * g->vol_f3[k] < rp.r_cut) { /* the cells of the candidate box would be too small */
			rs->error = PPI_E_GRID;
			rs->tries[7]++;
			return;
		}
	}
	g->vol_dir = PPI_LX_DIR;
	g->vol_mask = 7;
	g->vol_V0 = g->vol_V1 = rs->V;
}

/* an accepted candidate box: the cell grid scales with the box, cell membership is unchanged */
__device__ void grid_scale_axis(ppi_grid *g, ppi_rstate *rs, int a) {
	const double f = g->vol_f3[a];
	rs->box[a] = g->vol_box3[a];
	g->w[a] *= f;
	g->shift[a] *= f;
	g->shiftf[a] = (float) g->shift[a];
	g->wf[a] = (float) g->w[a];
	g->inv_w[a] = 1.0 / g->w[a];
	g->inv_L[a] = 1.0 / rs->box[a];
	g->inv_wf[a] = (float) g->inv_w[a];
	g->inv_Lf[a] = (float) g->inv_L[a];
	g->Lf[a] = (float) rs->box[a];
}

__global__ void k_vol_decide(ppi_dev d, long long sweep) {
	grid_dep_wait();
	grid_dep_release();
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	sweep = ctr_index(sweep, sweep < 0 ? d.ctr->sweep : 0);
	const ppi_rparams &rp = d.rp[r];
	ppi_grid *g = d.grid + r;
	ppi_rstate *rs = d.rs + r;
	if(g->vol_dir < 0) return;
	const long long nb_new = rs->vol_bonds / 2; /* every bonded pair was counted from both sides */
	const double dE = (double) (rs->bonds - nb_new);
	const U4 u = rng(rp, sweep, r, TAG_VOL, 0, 1);
	if(g->vol_dir == PPI_LX_DIR) {
		rs->tries[7]++;
		/* MC.c:562 accepts with min(1, exp(+dE / T)); lx_move = 2 takes the Boltzmann factor exp(-dE / T) */
		const double arg = (rp.lx_move == 2 ? -dE : dE) / rp.T;
		if(!rs->vol_overlap && u01d(u.x, u.y) < exp(arg)) {
			rs->vol_accept = 1;
			d.ctr->vol_any = 1;
			rs->bonds = nb_new;
			rs->accepted[7]++;
			for(int a = 0; a < 3; a++) grid_scale_axis(g, rs, a);
		}
		return;
	}
	rs->tries[6]++;
	double dV = g->vol_V1 - g->vol_V0;
	double arg = -(rp.P * dV + dE) / rp.T + (double) (rp.N + 1) * log(g->vol_f); /* MC.c:497-498 */
	if(!rs->vol_overlap && u01d(u.x, u.y) < exp(arg)) {
		rs->vol_accept = 1;
		d.ctr->vol_any = 1;
		rs->V = g->vol_V1;
		rs->bonds = nb_new;
		rs->accepted[6]++;
		grid_scale_axis(g, rs, g->vol_dir);
	}
}

__global__ void k_vol_apply(ppi_dev d) {
	grid_dep_wait();
	grid_dep_release();
	if(!d.ctr->vol_any) return; /* every replica rejected its candidate box: nothing to rescale */
	for(int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.ntot; k += gridDim.x * blockDim.x) {
		/* canonical positions (slot k): p->r[a] *= rescale_factor (MC.c:477, MC.c:541-544) */
		int r = d.rep[k];
		if(d.rs[r].vol_accept) {
			const ppi_grid &g = d.grid[r];
			double *rec = d.rec + (size_t) k * PPI_REC;
			for(int a = 0; a < 3; a++)
				if((g.vol_mask >> a) & 1) rec[a] = __dmul_rn(rec[a], g.vol_f3[a]);
		}
		/* working record (sorted position k) */
		int gc = __float_as_int(d.sori[3 * (size_t) k + 2].z);
		int r2 = d.cell_rep[gc];
		if(d.rs[r2].vol_accept) {
			const ppi_grid &g = d.grid[r2];
			float4 a = d.spos[k];
			a.x *= g.vol_ff3[0];
			a.y *= g.vol_ff3[1];
			a.z *= g.vol_ff3[2];
			d.spos[k] = a;
		}
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* gram_schmidt, reorder, export                                                                    */
/* ------------------------------------------------------------------------------------------------ */
__device__ void normalize64(double *v) {
	double norm = __dsqrt_rn(scalar64(v, v));
	v[0] = __ddiv_rn(v[0], norm);
	v[1] = __ddiv_rn(v[1], norm);
	v[2] = __ddiv_rn(v[2], norm);
}

/* gram_schmidt (utils.c:91-113) on the orientation rows R = R0 . Q(q), with explicitly rounded
 * operations; the result becomes the new R0 and q the identity */
__global__ void k_gram_schmidt(ppi_dev d, int first, int count) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= count) return;
	double *rec = d.rec + (size_t) (first + k) * PPI_REC;
	double R[9];
	orient64(rec + PPI_R0, rec + PPI_Q, R);
	double v1[3] = { R[0], R[1], R[2] }, v2[3] = { R[3], R[4], R[5] }, v3[3] = { R[6], R[7], R[8] };
	double b1 = __ddiv_rn(scalar64(v2, v1), scalar64(v1, v1));
	for(int i = 0; i < 3; i++) v2[i] = __dsub_rn(v2[i], __dmul_rn(b1, v1[i]));
	double v3_v1 = scalar64(v3, v1), v3_v2 = scalar64(v3, v2), v2n = scalar64(v2, v2);
	b1 = __ddiv_rn(v3_v1, scalar64(v1, v1));
	double b2 = __ddiv_rn(v3_v2, v2n);
	for(int i = 0; i < 3; i++) v3[i] = __dsub_rn(v3[i], __dadd_rn(__dmul_rn(b1, v1[i]), __dmul_rn(b2, v2[i])));
	normalize64(v1);
	normalize64(v2);
	normalize64(v3);
	for(int i = 0; i < 3; i++) {
		rec[PPI_R0 + i] = v1[i];
		rec[PPI_R0 + 3 + i] = v2[i];
		rec[PPI_R0 + 6 + i] = v3[i];
	}
	rec[PPI_Q] = 1.0;
	rec[PPI_Q + 1] = 0.0;
	rec[PPI_Q + 2] = 0.0;
	rec[PPI_Q + 3] = 0.0;
}

/* physical reorder of the canonical state into the current cell order (locality of the FP64 updates) */
__global__ void k_gather(ppi_dev d) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= d.ntot) return;
	int s = __float_as_int(d.sori[3 * (size_t) k + 2].w);
	const double2 *src = (const double2 *) (d.rec + (size_t) s * PPI_REC);
	double2 *dst = (double2 *) (d.tmp_rec + (size_t) k * PPI_REC);
#pragma unroll
	for(int j = 0; j < PPI_REC / 2; j++) dst[j] = src[j];
	d.tmp_id[k] = d.id[s];
	d.sori[3 * (size_t) k + 2].w = __int_as_float(k);
}

/* x y z R00..R22 of slots [first, first + count) into tmp_rec (12 doubles each) */
__global__ void k_export(ppi_dev d, int first, int count) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= count) return;
	const double *rec = d.rec + (size_t) (first + k) * PPI_REC;
	double *o = d.tmp_rec + (size_t) k * 12;
	o[0] = rec[0];
	o[1] = rec[1];
	o[2] = rec[2];
	orient64(rec + PPI_R0, rec + PPI_Q, o + 3);
}

/* ------------------------------------------------------------------------------------------------ */
/* grand canonical and successive-umbrella-sampling insertions and removals (MC_add_remove)          */
/* ------------------------------------------------------------------------------------------------ */
/* One CTA per GC / SUS replica makes `attempts` attempts one after the other, as MC_add_remove
 * (MC.c:342-448) does: with probability 1/2 an insertion at a uniform position with a uniform random
 * orientation, accepted with min(1, exp(-dE / T) z V / (N + 1)), otherwise the removal of a uniformly
 * chosen particle, accepted with min(1, exp(-dE / T) N / (V z)); an insertion into a full system is an
 * error for GC (the reference stops, "increase GC_N_max") and a non-attempt for SUS, as is a removal at
 * N_min. The replica's particles stay in slots p0 .. p0 + N - 1: an insertion takes slot p0 + N, a removal
 * moves the particle of the last slot into the freed one, and the particle with the highest index takes
 * the removed particle's index (the reference's renumbering). The energy of the probe is exact: every
 * live particle within an FP32 pre-filter radius r_cut + 0.05 goes through interact64 (MC_would_interact
 * with the probe as p). The caller re-sorts the cells afterwards. SUS adds one histogram count of N after
 * every attempt (MC.c:50). */
#define TAG_EXCH 9u
#define EXCH_B 256

/* sum (orbit = 0) or bitwise or (orbit = 1) of v over the CTA; every thread of the CTA calls it */
__device__ __forceinline__ int block_sum_or(int v, int *ws, int orbit) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	v = orbit ? (int) __reduce_or_sync(0xffffffffu, (unsigned) v) : __reduce_add_sync(0xffffffffu, v);
	__syncthreads();
	if(lane == 0) ws[warp] = v;
	__syncthreads();
	int t = 0;
	for(int w = 0; w < (int) (blockDim.x >> 5); w++) t = orbit ? (t | ws[w]) : t + ws[w];
	__syncthreads();
	return t;
}

/* rotation matrix (rows) of the uniform random unit quaternion built from three uniforms (Shoemake 1992) */
__device__ __forceinline__ void uniform_rotation64(double u1, double u2, double u3, double *R) {
	const double a = sqrt(1.0 - u1), b = sqrt(u1);
	const double t2 = 6.283185307179586 * u2, t3 = 6.283185307179586 * u3;
	const double q[4] = { b * cos(t3), a * sin(t2), a * cos(t2), b * sin(t3) }; /* (w, x, y, z) */
	quatmat64(q, R);
}

__global__ void __launch_bounds__(EXCH_B) k_exchange(ppi_dev d, long long step, int attempts) {
	const int r = blockIdx.x;
	ppi_rparams *rp = d.rp + r;
	ppi_rstate *rs = d.rs + r;
	if(rp->ensemble != 1 && rp->ensemble != 3) return;
	__shared__ double s_r[3], s_R[9];
	__shared__ int s_ws[EXCH_B / 32], s_t, s_dn;
	const int tid = threadIdx.x;
	const int p0 = rp->p0, gc = rp->ensemble == 1;
	const double box[3] = { rs->box[0], rs->box[1], rs->box[2] };
	const double V = rs->V, z = rp->activity, T = rp->T;
	const float rf2 = (float) ((rp->r_cut + 0.05) * (rp->r_cut + 0.05));
	const float Lf[3] = { (float) box[0], (float) box[1], (float) box[2] }, iLf[3] = { 1.f / Lf[0], 1.f / Lf[1], 1.f / Lf[2] };
	int n = rs->n_live;
	if(tid == 0) s_dn = 0;
	for(int a = 0; a < attempts; a++) {
		const U4 u0 = rng(*rp, step, r, TAG_EXCH, (uint32_t) a, 0u), u1 = rng(*rp, step, r, TAG_EXCH, (uint32_t) a, 1u);
		const bool add = u01d(u0.x, u0.y) < 0.5;
		const double U = u01d(u0.z, u0.w);
		int skip = 0, probe = -1;
		if(add) {
			if(n == rp->n_max) {
				skip = 1;
				if(gc) {
					if(tid == 0) rs->error = PPI_E_GCFULL;
					break;
				}
			}
			else if(tid == 0) { /* the candidate: uniform position, uniform orientation */
				const U4 u2 = rng(*rp, step, r, TAG_EXCH, (uint32_t) a, 2u), u3 = rng(*rp, step, r, TAG_EXCH, (uint32_t) a, 3u);
				s_r[0] = u01d(u1.x, u1.y) * box[0];
				s_r[1] = u01d(u1.z, u1.w) * box[1];
				s_r[2] = u01d(u2.x, u2.y) * box[2];
				uniform_rotation64(u01d(u2.z, u2.w), u01d(u3.x, u3.y), u01d(u3.z, u3.w), s_R);
			}
		}
		else if(n == rp->n_min) skip = 1;
		else {
			const int k = (int) (u01d(u1.x, u1.y) * n);
			probe = p0 + (k < n ? k : n - 1);
			if(tid == 0) {
				const double *rec = d.rec + (size_t) probe * PPI_REC;
				s_r[0] = rec[0];
				s_r[1] = rec[1];
				s_r[2] = rec[2];
				orient64(rec + PPI_R0, rec + PPI_Q, s_R);
			}
		}
		if(!skip) {
			__syncthreads();
			/* the probe's bonds and overlaps with every other live particle; for a removal also the slot
			 * of the particle with the highest index */
			int nb = 0, ov = 0;
			const float px = (float) s_r[0], py = (float) s_r[1], pz = (float) s_r[2];
			for(int j = tid; j < n; j += EXCH_B) {
				const int q = p0 + j;
				if(!add && d.id[q] == n - 1) s_t = q;
				if(q == probe) continue;
				const double *rec = d.rec + (size_t) q * PPI_REC;
				float dx = (float) rec[0] - px, dy = (float) rec[1] - py, dz = (float) rec[2] - pz;
				dx -= Lf[0] * rintf(dx * iLf[0]);
				dy -= Lf[1] * rintf(dy * iLf[1]);
				dz -= Lf[2] * rintf(dz * iLf[2]);
				if(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) >= rf2) continue;
				double Rq[9];
				orient64(rec + PPI_R0, rec + PPI_Q, Rq);
				const int res = interact64(s_r, s_R, rec, Rq, rp->base, box, rp->sqr_rcut, rp->cosmax, nullptr, nullptr, nullptr);
				nb += res == 1;
				ov |= res == -1;
			}
			nb = block_sum_or(nb, s_ws, 0);
			ov = block_sum_or(ov, s_ws, 1);
			if(tid == 0) {
				if(add) {
					rs->tries[2]++; /* ADD (defs.h:14) */
					const double acc = exp((double) nb / T) * z * V / (n + 1.);
					if(!ov && U < acc) {
						const int slot = p0 + n;
						double *rec = d.rec + (size_t) slot * PPI_REC;
						rec[0] = s_r[0];
						rec[1] = s_r[1];
						rec[2] = s_r[2];
						rec[PPI_Q] = 1.0;
						rec[PPI_Q + 1] = rec[PPI_Q + 2] = rec[PPI_Q + 3] = 0.0;
						for(int k = 0; k < 9; k++) rec[PPI_R0 + k] = s_R[k];
						d.id[slot] = n;
						rs->bonds += nb;
						rs->accepted[2]++;
						s_dn = 1;
					}
				}
				else {
					rs->tries[3]++; /* REMOVE (defs.h:15) */
					const double acc = exp(-(double) nb / T) * n / (V * z);
					if(U < acc) {
						const int last = p0 + n - 1;
						d.id[s_t] = d.id[probe]; /* the highest index takes the removed one's */
						if(probe != last) {
							double *dst = d.rec + (size_t) probe * PPI_REC;
							const double *src = d.rec + (size_t) last * PPI_REC;
							for(int k = 0; k < PPI_REC; k++) dst[k] = src[k];
							d.id[probe] = d.id[last];
						}
						rs->bonds -= nb;
						rs->accepted[3]++;
						s_dn = -1;
					}
				}
			}
			__syncthreads();
			n += s_dn; /* +1 inserted, -1 removed, 0 rejected */
			__syncthreads();
			if(tid == 0) s_dn = 0;
		}
		if(!gc && tid == 0) atomicAdd(d.sus_hist + (n - rp->n_min), 1ull); /* MC.c:50 */
		__syncthreads();
	}
	if(tid == 0) {
		rs->n_live = n;
		rp->N = n;
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* aggregation-volume-bias moves (Dynamics = 2, AVBMC_dynamics)                                      */
/* ------------------------------------------------------------------------------------------------ */
/* One CTA per AVB replica makes its AVB attempts one after the other, as AVBMC_dynamics (avb.c:77-186)
 * does for the fraction 1 - avb_p of the reference's attempts (the roto-translations of the other
 * fraction are the checkerboard rounds): a receiver drawn uniformly and its bonded partners indexed by
 * its bonding patch (_set_neighbours, avb.c:43-75); with probability 1/2 a particle outside its bonding
 * volume is placed inside it (place_inside_vbonding, utils.c:52-76) and accepted with
 * min(1, exp(-dE / T) (N - n - 1) V_in / ((n + 1) V_out)); otherwise one of its n partners goes to a
 * uniform position and orientation that does not bond to it, accepted with
 * min(1, exp(-dE / T) n V_out / ((N - n) V_in)). Neighbourhoods come from linked cells of edge >= r_cut
 * (cells.c:17-63) built from the FP64 state at the start of the batch and kept current as particles
 * move; every pair is decided in FP64 with the reference's operation order, so the tracked energy stays
 * exact. The caller re-sorts the engine's cells after the batch. */
#define AVB_B 64
#define TAG_AVB 10u
#define AVB_DRAWS 4096 /* draws a rejection loop may take before the batch stops with an error */

/* successive 53-bit uniforms of one attempt from its own Philox counter (item = attempt) */
struct AvbRng {
	const ppi_rparams *rp;
	long long step;
	int r;
	uint32_t item, sub;
	U4 u;
	int k;
	__device__ double next() {
		if(k == 0) {
			u = rng(*rp, step, r, TAG_AVB, item, sub++);
			k = 2;
		}
		k--;
		return k ? u01d(u.x, u.y) : u01d(u.z, u.w);
	}
};

/* cells_fill_and_get_idx_from_vector (cells.c:43-49) */
__device__ __forceinline__ int avb_cell_of(const double *r, const double *box, const int *ns, int *idx) {
#pragma unroll
	for(int a = 0; a < 3; a++) {
		const double f = r[a] / box[a];
		const int i = (int) ((f - floor(f)) * (1. - DBL_EPSILON) * ns[a]);
		idx[a] = i < 0 ? 0 : (i >= ns[a] ? ns[a] - 1 : i); /* [0, ns) for every finite position already */
	}
	return (idx[0] * ns[1] + idx[1]) * ns[2] + idx[2];
}

/* MC_would_interact (MC.c:232-266) with the reference's operation order for probe p at (pr, pR) and q at
 * qr, whose orientation is qR or, when qR is null, R0 . Q(q) of its record qrec: -1 overlap, 0 no bond,
 * 1 bond; *pa receives p's bonding patch (the first whose cosine passes, the reference's p_patch) */
__device__ __noinline__ int avb_pair(const double *pr, const double *pR, const double *qr, const double *qrec, const double *qR, const ppi_rparams &rp, const double *box,
		int *pa) {
	double d[3];
#pragma unroll 1
	for(int k = 0; k < 3; k++) {
		d[k] = __dsub_rn(qr[k], pr[k]);
		d[k] = __dsub_rn(d[k], __dmul_rn(box[k], rint(__ddiv_rn(d[k], box[k]))));
	}
	const double dist2 = scalar64(d, d);
	if(dist2 < 1.) return -1;
	if(!(dist2 < rp.sqr_rcut)) return 0;
	double Rq[9];
	if(qR == nullptr) orient64(qrec + PPI_R0, qrec + PPI_Q, Rq);
	else
		for(int k = 0; k < 9; k++) Rq[k] = qR[k];
	const double norm = __dsqrt_rn(dist2);
	d[0] = __ddiv_rn(d[0], norm);
	d[1] = __ddiv_rn(d[1], norm);
	d[2] = __ddiv_rn(d[2], norm);
	double P[3];
	int first = -1, qok = 0;
#pragma unroll 1
	for(int a = 0; a < 4; a++) {
		patch64(pR, rp.base[a], P);
		if(first < 0 && scalar64(d, P) > rp.cosmax) first = a;
	}
#pragma unroll 1
	for(int b = 0; b < 4; b++) {
		patch64(Rq, rp.base[b], P);
		if(-scalar64(d, P) > rp.cosmax) qok = 1;
	}
	if(first >= 0 && qok) {
		*pa = first;
		return 1;
	}
	return 0;
}

struct AvbShared {
	double pr[3], pR[9];   /* the probe of the next scan */
	double nr[3], nR[9];   /* the moving particle's candidate state */
	int nb, ov, nbp[4];    /* scan results: bonds, overlap, partners by the probe's patch */
	int rec, p, nn, skip, nb_old, in;
};

/* the 27 cells around S.pr (the reference's MC_energy walk, MC.c:272-309): the probe (S.pr, S.pR) against
 * every particle there but slot offset `self`; thread t < 27 walks cell t. Every thread of the CTA calls
 * it after S.nb, S.ov (and S.nbp) were cleared. */
__device__ void avb_scan(const ppi_dev &d, const ppi_rparams &rp, const double *box, const int *ns, AvbShared &S, int self, bool partners) {
	const int t = threadIdx.x;
	if(t < 27) {
		int idx[3];
		avb_cell_of(S.pr, box, ns, idx);
		const int cx = (idx[0] + t % 3 - 1 + ns[0]) % ns[0], cy = (idx[1] + (t / 3) % 3 - 1 + ns[1]) % ns[1], cz = (idx[2] + t / 9 - 1 + ns[2]) % ns[2];
		int q = d.avb_head[rp.avb_head0 + (cx * ns[1] + cy) * ns[2] + cz];
		for(int guard = 0; q != -1 && guard < rp.N; guard++) {
			if(q != self) {
				const double *qrec = d.rec + (size_t) (rp.p0 + q) * PPI_REC;
				int pa = 0;
				const int res = avb_pair(S.pr, S.pR, qrec, qrec, nullptr, rp, box, &pa);
				if(res == -1) S.ov = 1;
				else if(res == 1) {
					atomicAdd(&S.nb, 1);
					if(partners) S.nbp[pa] = q;
				}
			}
			q = d.avb_next[rp.p0 + q];
		}
	}
	__syncthreads();
}

/* random_vector_on_sphere (utils.c:115-131), Marsaglia (1972); false when the draws ran out */
__device__ bool avb_sphere(AvbRng &g, double *res) {
	for(int k = 0; k < 64; k++) {
		const double r1 = 1. - 2. * g.next(), r2 = 1. - 2. * g.next(), sq = r1 * r1 + r2 * r2;
		if(sq < 1.) {
			const double h = 2. * sqrt(1. - sq);
			res[0] = r1 * h;
			res[1] = r2 * h;
			res[2] = 1. - 2. * sq;
			return true;
		}
	}
	return false;
}

/* get_rotation_matrix (utils.c:186-202) */
__device__ void avb_rot(const double *a, double t, double *m) {
	double st, ct;
	sincos(t, &st, &ct);
	const double uct = 1. - ct;
	m[0] = a[0] * a[0] + (1. - a[0] * a[0]) * ct;
	m[1] = a[0] * a[1] * uct - a[2] * st;
	m[2] = a[0] * a[2] * uct + a[1] * st;
	m[3] = a[0] * a[1] * uct + a[2] * st;
	m[4] = a[1] * a[1] + (1. - a[1] * a[1]) * ct;
	m[5] = a[1] * a[2] * uct - a[0] * st;
	m[6] = a[0] * a[2] * uct - a[1] * st;
	m[7] = a[1] * a[2] * uct + a[0] * st;
	m[8] = a[2] * a[2] + (1. - a[2] * a[2]) * ct;
}

__device__ void avb_matvec(const double *m, const double *v, double *o) {
	for(int i = 0; i < 3; i++) o[i] = m[3 * i] * v[0] + m[3 * i + 1] * v[1] + m[3 * i + 2] * v[2];
}

__device__ void avb_matmul(const double *m, const double *n, double *o) {
	for(int i = 0; i < 3; i++)
		for(int j = 0; j < 3; j++) o[3 * i + j] = m[3 * i] * n[j] + m[3 * i + 1] * n[3 + j] + m[3 * i + 2] * n[6 + j];
}

__device__ void avb_normalize(double *v) {
	const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
	v[0] /= n;
	v[1] /= n;
	v[2] /= n;
}

/* gram_schmidt (utils.c:91-113) */
__device__ void avb_gram_schmidt(double *v1, double *v2, double *v3) {
	const double n1 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
	double b1 = (v2[0] * v1[0] + v2[1] * v1[1] + v2[2] * v1[2]) / n1;
	for(int k = 0; k < 3; k++) v2[k] -= b1 * v1[k];
	const double n2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
	b1 = (v3[0] * v1[0] + v3[1] * v1[1] + v3[2] * v1[2]) / n1;
	const double b2 = (v3[0] * v2[0] + v3[1] * v2[1] + v3[2] * v2[2]) / n2;
	for(int k = 0; k < 3; k++) v3[k] -= b1 * v1[k] + b2 * v2[k];
	avb_normalize(v1);
	avb_normalize(v2);
	avb_normalize(v3);
}

__device__ double avb_det(const double *m) {
	return m[0] * m[4] * m[8] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[2] * m[4] * m[6] - m[0] * m[5] * m[7] - m[1] * m[3] * m[8];
}

/* set_orientation_around_vector (utils.c:225-270): orient = B . orient, B's third column -v turned by t
 * about a random axis perpendicular to v */
__device__ bool avb_orient_around(AvbRng &g, const double *v, double *orient, double t) {
	double y_tmp[3] = { -v[0], -v[1], -v[2] }, z[3], w_tmp[3];
	if(!avb_sphere(g, z) || !avb_sphere(g, w_tmp)) return false;
	avb_gram_schmidt(y_tmp, z, w_tmp);
	double m[9], y[3], w[3];
	avb_rot(z, t, m);
	avb_matvec(m, y_tmp, y);
	avb_matvec(m, w_tmp, w);
	double B[9] = { z[0], w[0], y[0], z[1], w[1], y[1], z[2], w[2], y[2] };
	if(avb_det(B) < 0.)
		for(int i = 0; i < 3; i++) {
			B[3 * i] = w[i];
			B[3 * i + 1] = z[i];
		}
	double old[9];
	for(int k = 0; k < 9; k++) old[k] = orient[k];
	avb_matmul(B, old, orient);
	return true;
}

/* place_inside_vbonding (utils.c:52-76): position nr and orientation nR inside the bonding volume of patch
 * tp of the particle at (rr, rR) */
__device__ bool avb_place_inside(const ppi_rparams &rp, AvbRng &g, const double *rr, const double *rR, int tp, double *nr, double *nR) {
	double m[9];
	avb_rot(rp.base[0], 2. * g.next() * 3.141592653589793, m);
	avb_matmul(rp.base_orient, m, nR);
	double dir[3], nv[3];
	patch64(rR, rp.base[tp], dir);
	if(!avb_sphere(g, nv)) return false; /* get_perpendicular_versor (utils.c:38-50) */
	const double vv = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2], rv = nv[0] * dir[0] + nv[1] * dir[1] + nv[2] * dir[2];
	for(int k = 0; k < 3; k++) nv[k] -= rv / vv * dir[k];
	avb_normalize(nv);
	const double theta = acos(rp.cosmax + (1. - rp.cosmax) * g.next());
	avb_rot(nv, theta, m);
	double tmp[3];
	avb_matvec(m, dir, tmp);
	for(int k = 0; k < 3; k++) dir[k] = tmp[k];
	avb_normalize(dir);
	const double theta2 = acos(rp.cosmax + (1. - rp.cosmax) * g.next());
	if(!avb_orient_around(g, dir, nR, theta2)) return false;
	const double dl = rp.r_cut - 1.;
	const double dist = pow(1. + g.next() * (dl * dl * dl + 3. * dl * dl + 3. * dl), 1. / 3.);
	for(int k = 0; k < 3; k++) nr[k] = dir[k] * dist + rr[k];
	return true;
}

__global__ void __launch_bounds__(AVB_B) k_avb(ppi_dev d, long long step, int steps) {
	const int r = blockIdx.x, tid = threadIdx.x;
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	if(rp.dynamics != 2) return;
	const int N = rp.N, p0 = rp.p0;
	const int attempts = rp.avb_per_step * steps;
	if(N < 2 || attempts <= 0) return;
	__shared__ AvbShared S;
	const double box[3] = { rs->box[0], rs->box[1], rs->box[2] };
	int ns[3];
	for(int a = 0; a < 3; a++) {
		int n = (int) floor(box[a] / rp.r_cut); /* cells_init (cells.c:17-37) */
		n = n < rp.avb_ncap[a] ? n : rp.avb_ncap[a];
		ns[a] = n < 3 ? 3 : n;
	}
	const int ncell = ns[0] * ns[1] * ns[2];
	/* linked cells of the live particles (cells_fill, cells.c:51-63); the order inside a cell does not
	 * change any outcome: bonds and overlaps are counted, and each patch bonds at most one partner */
	for(int c = tid; c < ncell; c += AVB_B) d.avb_head[rp.avb_head0 + c] = -1;
	__syncthreads();
	for(int i = tid; i < N; i += AVB_B) {
		int idx[3];
		const int c = avb_cell_of(d.rec + (size_t) (p0 + i) * PPI_REC, box, ns, idx);
		d.avb_cell[p0 + i] = c;
		d.avb_next[p0 + i] = atomicExch(&d.avb_head[rp.avb_head0 + c], i);
	}
	__syncthreads();
	AvbRng g;
	for(int a = 0; a < attempts; a++) {
		if(tid == 0) {
			g.rp = &rp;
			g.step = step;
			g.r = r;
			g.item = (uint32_t) a;
			g.sub = 0u;
			g.k = 0;
			int rec = (int) (g.next() * N);
			S.rec = rec < N ? rec : N - 1;
			const double *q = d.rec + (size_t) (p0 + S.rec) * PPI_REC;
			for(int k = 0; k < 3; k++) S.pr[k] = q[k];
			orient64(q + PPI_R0, q + PPI_Q, S.pR);
			S.nb = S.ov = 0;
			for(int k = 0; k < 4; k++) S.nbp[k] = -1;
			rs->tries[1]++; /* AVB (defs.h:13) */
		}
		__syncthreads();
		avb_scan(d, rp, box, ns, S, S.rec, true); /* _set_neighbours of the receiver */
		if(tid == 0) {
			S.nn = S.nb;
			S.skip = 0;
			const double rr[3] = { S.pr[0], S.pr[1], S.pr[2] };
			double rR[9];
			for(int k = 0; k < 9; k++) rR[k] = S.pR[k];
			S.in = g.next() > 0.5;
			if(S.in) { /* into the receiver's bonding volume */
				if(S.nn == N - 1) S.skip = 1;
				else {
					int p = -1;
					for(int k = 0; k < AVB_DRAWS && p < 0; k++) {
						int c = (int) (g.next() * N);
						c = c < N ? c : N - 1;
						if(c != S.rec && c != S.nbp[0] && c != S.nbp[1] && c != S.nbp[2] && c != S.nbp[3]) p = c;
					}
					int tp = (int) (g.next() * 4);
					tp = tp < 4 ? tp : 3;
					if(p < 0 || !avb_place_inside(rp, g, rr, rR, tp, S.nr, S.nR)) {
						rs->error = PPI_E_AVB;
						S.skip = 2;
					}
					S.p = p;
				}
			}
			else { /* a partner out of it */
				if(S.nn == 0) S.skip = 1;
				else {
					int k = (int) (g.next() * S.nn), cn = 0, ci = 0;
					while(cn <= k && ci < 4) {
						if(S.nbp[ci] != -1) cn++;
						ci++;
					}
					S.p = S.nbp[ci - 1];
					if(S.p < 0) S.skip = 1; /* only if two partners shared a patch, which overlaps forbid */
					int tries = 0, pa = 0;
					for(; tries < AVB_DRAWS; tries++) {
						for(int c = 0; c < 3; c++) S.nr[c] = g.next() * box[c];
						const double u1 = g.next(), u2 = g.next(), u3 = g.next();
						uniform_rotation64(u1, u2, u3, S.nR);
						if(avb_pair(rr, rR, S.nr, nullptr, S.nR, rp, box, &pa) != 1) break;
					}
					if(tries == AVB_DRAWS) {
						rs->error = PPI_E_AVB;
						S.skip = 2;
					}
				}
			}
			if(!S.skip) {
				/* the mover's current state is the next probe; its candidate position is r + (new_r - r)
				 * (MC_rototraslate_particle, MC.c:208-230) */
				const double *q = d.rec + (size_t) (p0 + S.p) * PPI_REC;
				for(int k = 0; k < 3; k++) {
					S.pr[k] = q[k];
					S.nr[k] = __dadd_rn(q[k], __dsub_rn(S.nr[k], q[k]));
				}
				orient64(q + PPI_R0, q + PPI_Q, S.pR);
			}
			S.nb = S.ov = 0;
		}
		__syncthreads();
		if(S.skip == 2) break;
		if(S.skip) continue;
		avb_scan(d, rp, box, ns, S, S.p, false); /* the mover's energy now */
		if(tid == 0) {
			S.nb_old = S.nb;
			for(int k = 0; k < 3; k++) S.pr[k] = S.nr[k];
			for(int k = 0; k < 9; k++) S.pR[k] = S.nR[k];
			S.nb = S.ov = 0;
		}
		__syncthreads();
		avb_scan(d, rp, box, ns, S, S.p, false); /* and at the candidate state */
		if(tid == 0) {
			const int n = S.nn;
			const double dE = -(double) (S.nb - S.nb_old);
			/* avb.c:116 (in) and avb.c:173 (out) */
			const double ratio = S.in ? (N - n - 1.) * rp.avb_vin / ((n + 1.) * rp.avb_vout) : (double) n * rp.avb_vout / ((N - n) * rp.avb_vin);
			if(!S.ov && g.next() < exp(-dE / rp.T) * ratio) {
				double *q = d.rec + (size_t) (p0 + S.p) * PPI_REC;
				for(int k = 0; k < 3; k++) q[k] = S.nr[k];
				q[PPI_Q] = 1.0;
				q[PPI_Q + 1] = q[PPI_Q + 2] = q[PPI_Q + 3] = 0.0;
				for(int k = 0; k < 9; k++) q[PPI_R0 + k] = S.nR[k];
				/* MC_change_cell (MC.c:180-206) on the batch's linked cells */
				int idx[3];
				const int c_new = avb_cell_of(S.nr, box, ns, idx), c_old = d.avb_cell[p0 + S.p];
				if(c_new != c_old) {
					int *h = d.avb_head + rp.avb_head0;
					if(h[c_old] == S.p) h[c_old] = d.avb_next[p0 + S.p];
					else {
						int w = h[c_old];
						for(int guard = 0; w != -1 && d.avb_next[p0 + w] != S.p && guard < N; guard++) w = d.avb_next[p0 + w];
						if(w != -1) d.avb_next[p0 + w] = d.avb_next[p0 + S.p];
					}
					d.avb_next[p0 + S.p] = h[c_new];
					h[c_new] = S.p;
					d.avb_cell[p0 + S.p] = c_new;
				}
				rs->bonds += S.nb - S.nb_old;
				rs->accepted[1]++;
			}
		}
		__syncthreads();
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* virtual-move Monte Carlo (Dynamics = 1, VMMC_dynamics)                                            */
/* ------------------------------------------------------------------------------------------------ */
/* One CTA per VMMC replica makes N cluster moves per MC step one after the other, as VMMC_dynamics
 * (vmmc.c:258-483) does for every attempt: a seed and a random translation (Disp_max) or rotation about the
 * seed (Theta_max); links to neighbours within the bonding range before and after the seed's virtual move
 * (_populate_possible_links, vmmc.c:148-229, with its image bookkeeping); links drawn at random, p
 * recruiting q with 1 - exp((E_old - E_p_moved) / T) and q agreeing with the ratio of the reverse virtual
 * move's probability (overlaps force the link); prelinked particles left outside reject the move, as does
 * a cluster reaching vmmc_max_cluster; an accepted move shifts the whole cluster. The orientations are made
 * canonical (R0 = R0 . Q(q), q = 1) at the start of the batch, so that the stored R0 is the orientation
 * matrix the moves rotate, as the reference's orientation field. Pair energies are the reference's FP64
 * test (explicitly rounded), so the tracked energy stays exact; the cluster energies use 27 threads, one
 * per neighbour cell; the rest of a move is one thread's sequential work. The caller re-sorts after the
 * batch. */
#define VM_B 64
#define TAG_VMMC 11u
#define VM_LINKS 16 /* links, prelinked and failed entries per particle (possible_links holds 16 N, vmmc.c:29) */

struct VmCtx {
	const ppi_dev *d;
	const ppi_rparams *rp;
	double box[3];
	int ns[3];
	int p0, N;
	int rot;
	double move[3], Rm[9];
	int nclust, nlinks, npre, nfail;
	int err;
};

__device__ __forceinline__ double *vm_rec(const VmCtx &c, int i) { return c.d->rec + (size_t) (c.p0 + i) * PPI_REC; }
__device__ __forceinline__ double *vm_old(const VmCtx &c, int i) { return c.d->vm_old + (size_t) (c.p0 + i) * 12; }

/* _store_dof / _restore_dof (vmmc.c:58-79): position and orientation (R0 with q = 1) */
__device__ void vm_store(const VmCtx &c, int i) {
	const double *r = vm_rec(c, i);
	double *o = vm_old(c, i);
	for(int k = 0; k < 3; k++) o[k] = r[k];
	for(int k = 0; k < 9; k++) o[3 + k] = r[PPI_R0 + k];
}

__device__ void vm_restore(const VmCtx &c, int i) {
	double *r = vm_rec(c, i);
	const double *o = vm_old(c, i);
	for(int k = 0; k < 3; k++) r[k] = o[k];
	for(int k = 0; k < 9; k++) r[PPI_R0 + k] = o[3 + k];
}

/* _pair_energy (vmmc.c:81-95): -1 bond, 0 otherwise; an overlap sets *ov */
__device__ double vm_pair_energy(const VmCtx &c, int p, int q, int *ov) {
	const double *a = vm_rec(c, p), *b = vm_rec(c, q);
	int pa = 0;
	const int res = avb_pair(a, a + PPI_R0, b, nullptr, b + PPI_R0, *c.rp, c.box, &pa);
	if(res == 1) return -1.;
	if(res == -1) *ov = 1;
	return 0.;
}

/* _move_particle (vmmc.c:231-256), after vm_store(i): the translation, or the rotation about the seed */
__device__ void vm_move(const VmCtx &c, int i) {
	double *r = vm_rec(c, i);
	if(!c.rot) {
		for(int k = 0; k < 3; k++) r[k] += c.move[k];
		return;
	}
	const int seed = c.d->vm_clust[c.p0];
	const double *sr = vm_rec(c, seed);
	const double dt[3] = { r[0] - sr[0], r[1] - sr[1], r[2] - sr[2] };
	double dr[3];
	avb_matvec(c.Rm, dt, dr);
	for(int k = 0; k < 3; k++) r[k] = sr[k] + dr[k];
	avb_matmul(c.Rm, vm_old(c, i) + 3, r + PPI_R0);
}

/* MC_change_cell (MC.c:180-206) on the batch's linked cells */
__device__ void vm_change_cell(const VmCtx &c, int i) {
	const ppi_dev &d = *c.d;
	int idx[3];
	const int cn = avb_cell_of(vm_rec(c, i), c.box, c.ns, idx), co = d.avb_cell[c.p0 + i];
	if(cn == co) return;
	int *h = d.avb_head + c.rp->avb_head0;
	if(h[co] == i) h[co] = d.avb_next[c.p0 + i];
	else {
		int w = h[co];
		for(int guard = 0; w != -1 && d.avb_next[c.p0 + w] != i && guard < c.N; guard++) w = d.avb_next[c.p0 + w];
		if(w != -1) d.avb_next[c.p0 + w] = d.avb_next[c.p0 + i];
	}
	d.avb_next[c.p0 + i] = h[cn];
	h[cn] = i;
	d.avb_cell[c.p0 + i] = cn;
}

__device__ void vm_drop_link(VmCtx &c, int k, int p, int q) {
	int *L = c.d->vm_links + 2 * (size_t) VM_LINKS * c.p0;
	L[2 * k] = L[2 * (c.nlinks - 1)];
	L[2 * k + 1] = L[2 * (c.nlinks - 1) + 1];
	c.nlinks--;
	int *cnt = c.d->vm_cnt + c.p0, *cp = c.d->vm_copies + c.p0;
	cnt[p]--;
	cnt[q]--;
	if(cnt[p] == 0) cp[p] = 0;
	if(cnt[q] == 0) cp[q] = 0;
}

/* _populate_possible_links (vmmc.c:148-229) for particle i at its current (real or virtual) position */
__device__ void vm_populate(VmCtx &c, int i, int *force_reject) {
	const ppi_dev &d = *c.d;
	int idx[3];
	const double *ri = vm_rec(c, i), *ro = vm_old(c, i);
	avb_cell_of(ri, c.box, c.ns, idx);
	int *L = d.vm_links + 2 * (size_t) VM_LINKS * c.p0, *cnt = d.vm_cnt + c.p0, *cp = d.vm_copies + c.p0, *in = d.vm_in + c.p0;
	for(int t = 0; t < 27; t++) {
		const int cx = (idx[0] + t / 9 - 1 + c.ns[0]) % c.ns[0], cy = (idx[1] + (t / 3) % 3 - 1 + c.ns[1]) % c.ns[1], cz = (idx[2] + t % 3 - 1 + c.ns[2]) % c.ns[2];
		int q = d.avb_head[c.rp->avb_head0 + (cx * c.ns[1] + cy) * c.ns[2] + cz];
		for(int guard = 0; q != -1 && guard < c.N; guard++) {
			if(q != i) {
				double *rq = vm_rec(c, q);
				double dist[3];
				for(int k = 0; k < 3; k++) {
					dist[k] = rq[k] - ri[k];
					dist[k] -= c.box[k] * rint(dist[k] / c.box[k]);
				}
				if(dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2] < c.rp->sqr_rcut) {
					if(c.nlinks >= VM_LINKS * c.N) { /* "VMMC: memory exhausted" (vmmc.c:176) */
						c.err = 1;
						*force_reject = 1;
						return;
					}
					double np[3];
					for(int k = 0; k < 3; k++) {
						dist[k] = rq[k] - ro[k];
						dist[k] -= c.box[k] * rint(dist[k] / c.box[k]);
						np[k] = ro[k] + dist[k];
					}
					if(cp[q] == 1 || in[q] == 1) {
						if(fabs(np[0] - rq[0]) > 1e-6 || fabs(np[1] - rq[1]) > 1e-6 || fabs(np[2] - rq[2]) > 1e-6) {
							*force_reject = 1;
							return;
						}
					}
					if(cp[q] == 0 && in[q] == 0) {
						for(int k = 0; k < 3; k++) rq[k] = np[k];
						cp[q] = 1;
					}
					const int n = c.nlinks, lo = i < q ? i : q, hi = i < q ? q : i;
					L[2 * n] = lo;
					L[2 * n + 1] = hi;
					c.nlinks++;
					cnt[i]++;
					cnt[q]++;
					for(int m = 0; m < c.nlinks - 1; m++)
						if(L[2 * m] == lo && L[2 * m + 1] == hi) {
							c.nlinks--;
							cnt[i]--;
							cnt[q]--;
							if(cnt[i] == 0) cp[i] = 0;
							if(cnt[q] == 0) cp[q] = 0;
							break;
						}
				}
			}
			q = d.avb_next[c.p0 + q];
		}
	}
}

struct VmShared {
	int fr, nb, ov, nclust, stop;
};

/* _compute_cluster_energy (vmmc.c:107-137): bonds between the cluster and the particles outside it, one
 * thread per neighbour cell of each member; every thread of the CTA calls it */
__device__ int vm_cluster_bonds(const VmCtx &c, VmShared &S) {
	const ppi_dev &d = *c.d;
	if(threadIdx.x == 0) {
		S.nb = 0;
		S.ov = 0;
	}
	__syncthreads();
	for(int m = 0; m < S.nclust; m++) {
		const int p = d.vm_clust[c.p0 + m];
		const int t = threadIdx.x;
		if(t < 27) {
			int idx[3];
			const double *rp = vm_rec(c, p);
			avb_cell_of(rp, c.box, c.ns, idx);
			const int cx = (idx[0] + t / 9 - 1 + c.ns[0]) % c.ns[0], cy = (idx[1] + (t / 3) % 3 - 1 + c.ns[1]) % c.ns[1], cz = (idx[2] + t % 3 - 1 + c.ns[2]) % c.ns[2];
			int q = d.avb_head[c.rp->avb_head0 + (cx * c.ns[1] + cy) * c.ns[2] + cz];
			int nb = 0, ov = 0;
			for(int guard = 0; q != -1 && guard < c.N; guard++) {
				if(d.vm_in[c.p0 + q] == 0) nb -= (int) vm_pair_energy(c, p, q, &ov);
				q = d.avb_next[c.p0 + q];
			}
			if(nb) atomicAdd(&S.nb, nb);
			if(ov) S.ov = 1;
		}
		__syncthreads();
	}
	return S.nb;
}

__global__ void __launch_bounds__(VM_B) k_vmmc(ppi_dev d, long long step, int steps) {
	const int r = blockIdx.x, tid = threadIdx.x;
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	if(rp.dynamics != 1) return;
	const int N = rp.N;
	if(N < 1) return;
	__shared__ VmShared S;
	VmCtx c;
	c.d = &d;
	c.rp = &rp;
	for(int a = 0; a < 3; a++) {
		c.box[a] = rs->box[a];
		int n = (int) floor(c.box[a] / rp.r_cut); /* cells_init (cells.c:17-37) */
		n = n < rp.avb_ncap[a] ? n : rp.avb_ncap[a];
		c.ns[a] = n < 3 ? 3 : n;
	}
	c.p0 = rp.p0;
	c.N = N;
	c.nclust = c.nlinks = c.npre = c.nfail = 0;
	c.err = 0;
	const int ncell = c.ns[0] * c.ns[1] * c.ns[2];
	for(int k = tid; k < ncell; k += VM_B) d.avb_head[rp.avb_head0 + k] = -1;
	__syncthreads();
	for(int i = tid; i < N; i += VM_B) {
		double *q = vm_rec(c, i);
		double R[9]; /* canonical orientation: R0 = R0 . Q(q), q = 1 (the same matrix every pass reads) */
		orient64(q + PPI_R0, q + PPI_Q, R);
		for(int k = 0; k < 9; k++) q[PPI_R0 + k] = R[k];
		q[PPI_Q] = 1.0;
		q[PPI_Q + 1] = q[PPI_Q + 2] = q[PPI_Q + 3] = 0.0;
		d.vm_cnt[c.p0 + i] = d.vm_copies[c.p0 + i] = d.vm_in[c.p0 + i] = 0;
		int idx[3];
		const int cc = avb_cell_of(q, c.box, c.ns, idx);
		d.avb_cell[c.p0 + i] = cc;
		d.avb_next[c.p0 + i] = atomicExch(&d.avb_head[rp.avb_head0 + cc], i);
	}
	__syncthreads();
	const long long moves = (long long) N * steps;
	int *clust = d.vm_clust + c.p0, *in = d.vm_in + c.p0, *cp = d.vm_copies + c.p0, *cnt = d.vm_cnt + c.p0;
	int *L = d.vm_links + 2 * (size_t) VM_LINKS * c.p0, *pre = d.vm_pre + (size_t) VM_LINKS * c.p0, *fail = d.vm_fail + (size_t) VM_LINKS * c.p0;
	AvbRng g;
	int nb_before = 0;
	for(long long m = 0; m < moves; m++) {
		if(tid == 0) {
			g.rp = &rp;
			g.step = step;
			g.r = r;
			g.item = (uint32_t) m;
			g.sub = 0u;
			g.k = 0;
			rs->tries[5]++; /* MOVE_VMMC (defs.h:17) */
			int fr = 0;
			c.nclust = 1;
			c.nfail = c.nlinks = c.npre = 0;
			int seed = (int) (g.next() * N);
			seed = seed < N ? seed : N - 1;
			in[seed] = 1;
			clust[0] = seed;
			if(g.next() < 0.5) {
				c.rot = 0;
				for(int k = 0; k < 3; k++) c.move[k] = (g.next() - 0.5) * rp.disp_max;
			}
			else {
				c.rot = 1;
				if(!avb_sphere(g, c.move)) {
					c.err = 1;
					fr = 1;
				}
				const double angle = g.next() * rp.theta_max;
				avb_rot(c.move, angle, c.Rm);
			}
			vm_store(c, seed);
			if(!fr) vm_populate(c, seed, &fr);
			if(!fr) {
				vm_move(c, seed);
				vm_populate(c, seed, &fr);
				vm_restore(c, seed);
			}
			while(c.nlinks > 0 && c.nclust < rp.vmmc_max_cluster && !fr) {
				int k = (int) (g.next() * c.nlinks);
				k = k < c.nlinks ? k : c.nlinks - 1;
				int p = L[2 * k], q = L[2 * k + 1];
				if(in[p] == 1 && in[q] == 1) {
					vm_drop_link(c, k, p, q);
					continue;
				}
				if(in[p] == 0) {
					const int t = q;
					q = p;
					p = t;
				}
				int ov = 0;
				const double E_old = vm_pair_energy(c, p, q, &ov);
				vm_store(c, p);
				vm_move(c, p);
				ov = 0;
				const double E_p = vm_pair_energy(c, p, q, &ov);
				vm_restore(c, p);
				const int force_prelink = ov;
				const double p1 = 1. - exp((1. / rp.T) * (E_old - E_p));
				if(force_prelink == 1 || p1 > g.next()) {
					vm_store(c, q);
					vm_move(c, q);
					ov = 0;
					const double E_q = vm_pair_energy(c, p, q, &ov);
					vm_restore(c, q);
					const int force_link = ov;
					double p2 = 1. - exp((1. / rp.T) * (E_old - E_q));
					if(p2 > 1.) p2 = 1.;
					if(force_link == 1 || (p2 / p1) > g.next()) {
						cp[q] = 0;
						in[q] = 1;
						clust[c.nclust++] = q;
						vm_store(c, q);
						vm_populate(c, q, &fr);
						if(fr) break;
						vm_move(c, q);
						vm_populate(c, q, &fr);
						vm_restore(c, q);
						if(fr) break;
					}
					else if(c.npre < VM_LINKS * N) pre[c.npre++] = q;
					else {
						c.err = 1;
						fr = 1;
						break;
					}
				}
				else if(c.nfail < VM_LINKS * N) fail[c.nfail++] = q;
				else {
					c.err = 1;
					fr = 1;
					break;
				}
				vm_drop_link(c, k, p, q);
			}
			if(c.nclust == rp.vmmc_max_cluster) fr = 1;
			for(int i = 0; i < c.npre; i++) {
				if(in[pre[i]] == 0) fr = 1;
				else cp[pre[i]] = 0;
			}
			S.fr = fr;
			S.nclust = c.nclust;
			S.stop = c.err;
		}
		__syncthreads();
		if(!S.fr) nb_before = vm_cluster_bonds(c, S);
		if(tid == 0) {
			if(!S.fr && S.ov) c.err = 1; /* assert(syst->overlap == 0), vmmc.c:436 */
			for(int i = 0; i < c.nclust && !S.fr; i++) {
				vm_store(c, clust[i]);
				vm_move(c, clust[i]);
				vm_change_cell(c, clust[i]);
			}
		}
		__syncthreads();
		int nb_after = 0;
		if(!S.fr) nb_after = vm_cluster_bonds(c, S);
		if(tid == 0) {
			if(!S.fr && S.ov) c.err = 1; /* vmmc.c:446 */
			if(S.fr)
				for(int i = 0; i < c.nclust; i++) vm_restore(c, clust[i]);
			else {
				rs->accepted[5]++;
				rs->bonds += nb_after - nb_before;
			}
			for(int i = 0; i < c.nclust; i++) {
				vm_change_cell(c, clust[i]);
				in[clust[i]] = 0;
			}
			for(int i = 0; i < c.nfail; i++) cp[fail[i]] = 0;
			for(int i = 0; i < c.nlinks; i++) {
				cp[L[2 * i]] = cp[L[2 * i + 1]] = 0;
				cnt[L[2 * i]] = cnt[L[2 * i + 1]] = 0;
			}
			if(c.err) rs->error = PPI_E_VMMC;
			S.stop = c.err;
		}
		__syncthreads();
		if(S.stop) break;
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* launchers                                                                                        */
/* ------------------------------------------------------------------------------------------------ */
static int g_sms = 0;

extern "C" int ppi_avb(const ppi_dev *d, long long step, int steps, cudaStream_t s, long long *nl) {
	k_avb<<<d->nrep, AVB_B, 0, s>>>(*d, step, steps);
	if(nl) *nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_vmmc(const ppi_dev *d, long long step, int steps, cudaStream_t s, long long *nl) {
	k_vmmc<<<d->nrep, VM_B, 0, s>>>(*d, step, steps);
	if(nl) *nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_sm_count(void) {
	if(g_sms == 0) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
		if(g_sms <= 0) g_sms = 1;
	}
	return g_sms;
}

/* one full wave of resident 128-thread CTAs of kernel f (the passes loop over their work) */
template <typename F>
static int resident_grid(F f, int *cache, int block = 128) {
	if(*cache == 0) {
		int nb = 0;
		if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, block, 0) != cudaSuccess || nb <= 0) nb = 1;
		*cache = nb * ppi_sm_count();
	}
	return *cache;
}

/* cached launch grids (one occupancy query each, made before any stream capture by ppi_prepare) */
static int g_col_audit = 0, g_col_fast = 0, g_learn_audit = 0, g_learn_fast = 0, g_vol_grid = 0, g_col_tl = 0, g_col_tla = 0;
static int g_a1 = 0, g_a4 = 0, g_f1 = 0, g_f4 = 0, g_f8 = 0, g_vol_list = 0, g_vol_pairs = 0;

static int pdl_enabled(void) {
	static int pdl = -1;
	if(pdl < 0) pdl = getenv("PPGPU_NO_PDL") ? 0 : 1;
	return pdl;
}

/* a launch with programmatic stream serialisation: the kernel may start before its predecessor completes
 * and waits for it (grid_dep_wait) before its first dependent access */
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
	cudaLaunchConfig_t cfg;
	memset(&cfg, 0, sizeof(cfg));
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(block);
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = pdl_enabled() ? 1 : 0;
	cudaLaunchKernelEx(&cfg, kern, args...);
}

extern "C" int ppi_resort(const ppi_dev *d, long long epoch, cudaStream_t s, long long *nl) {
	float4 *tmp = (float4 *) d->tmp_rec; /* ntot float4 fit in the reorder scratch */
	cudaMemsetAsync(d->cell_count, 0, sizeof(int) * (size_t) d->total_cells, s);
	cudaMemsetAsync(d->ccount, 0, sizeof(int) * 9, s); /* the 8 colour counts and k_scan's ticket */
	k_grid<<<(d->nrep + 1) / 2, 64, 0, s>>>(*d, epoch); /* a warp per replica */
	/* the rest of the sort is one chain of kernels, each launch overlapping its predecessor's tail
	 * (programmatic dependent launch; every kernel waits before its first access) */
	int nb = (d->ntot + 255) / 256;
	if(nb > 0) launch_pdl(k_assign, nb, 256, s, *d, tmp);
	int sb = (d->total_cells + SCAN_TILE - 1) / SCAN_TILE;
	launch_pdl(k_scan, sb, SCAN_B, s, (const int *) d->cell_count, d->cell_part, d->scan_aux, d->ccount + 8, d->cell_start + d->total_cells, d->total_cells);
	if(nb > 0) launch_pdl(k_scatter, nb, 256, s, *d, (const float4 *) tmp);
	launch_pdl(k_cellfin, (d->total_cells + CELLFIN_B - 1) / CELLFIN_B, CELLFIN_B, s, *d);
	*nl += 3 + (nb > 0 ? 2 : 0);
	return (int) cudaGetLastError();
}

static int lanes_of(const ppi_dev *d) { return d->lanes == 8 ? 8 : PPI_DEFAULT_LANES; }

/* the 8 colour launches of a round; colours 1..7 with programmatic stream serialisation (their proposals
 * overlap the previous colour's tail, see grid_dep_wait) */
template <typename K>
static void launch_round(K kern, int grid, int block, size_t smem, const ppi_dev *d, long long round, const int *colours, cudaStream_t s) {
	const int pdl = pdl_enabled();
	for(int ci = 0; ci < 8; ci++) {
		cudaLaunchConfig_t cfg;
		memset(&cfg, 0, sizeof(cfg));
		cfg.gridDim = dim3(grid);
		cfg.blockDim = dim3(block);
		cfg.dynamicSmemBytes = smem;
		cfg.stream = s;
		cudaLaunchAttribute at[1];
		at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
		at[0].val.programmaticStreamSerializationAllowed = 1;
		cfg.attrs = at;
		cfg.numAttrs = (ci > 0 && pdl) ? 1 : 0;
		cudaLaunchKernelEx(&cfg, kern, *d, round, colours[ci]);
	}
}

extern "C" int ppi_nlist(const ppi_dev *d, cudaStream_t s, long long *nl) {
	if(d->ntot <= 0 || d->nl_k <= 0) return 0;
	launch_pdl(k_nlist, (d->ntot + NL_B - 1) / NL_B, NL_B, s, *d); /* k_grid zeroed its counters */
	*nl += 1;
	return (int) cudaGetLastError();
}

/* the persistent round kernel's grid: every CTA resident (cooperative launch); 0 if it cannot run */
static int g_round_grid = -1;
static int round_grid(void) {
	if(g_round_grid < 0) {
		const int smem = (int) (sizeof(RoundSmem) * KR_WARPS);
		int nb = 0;
		if(cudaFuncSetAttribute(k_round, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
				cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_round, 32 * KR_WARPS, smem) != cudaSuccess)
			nb = 0;
		cudaGetLastError();
		g_round_grid = nb * ppi_sm_count();
	}
	return g_round_grid;
}

/* one plain round over the lists as one cooperative launch of k_round (the barrier counters cleared first) */
static int launch_persistent_round(const ppi_dev *d, long long round, const int *colours, cudaStream_t s) {
	int packed = 0;
	for(int ci = 0; ci < 8; ci++) packed |= (colours[ci] & 7) << (3 * ci);
	cudaMemsetAsync(d->gbar, 0, 9 * sizeof(int), s); /* the arrival counter and the colours' work counters (not the error word) */
	cudaLaunchConfig_t cfg;
	memset(&cfg, 0, sizeof(cfg));
	cfg.gridDim = dim3(round_grid());
	cfg.blockDim = dim3(32 * KR_WARPS);
	cfg.dynamicSmemBytes = sizeof(RoundSmem) * KR_WARPS;
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeCooperative;
	at[0].val.cooperative = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return (int) cudaLaunchKernelEx(&cfg, k_round, *d, round, packed);
}

extern "C" int ppi_round(const ppi_dev *d, long long round, const int *colours, int audit, int use_nl, cudaStream_t s, long long *nl) {
	const int aud = audit || d->audit_any;
	if(use_nl && d->nl_k > 0 && !aud && d->persist && d->gbar && round_grid() > 0) {
		const int rc = launch_persistent_round(d, round, colours, s);
		*nl += 1;
		return rc ? rc : (int) cudaGetLastError();
	}
	if(use_nl && d->nl_k > 0 && aud) launch_round(k_colour<MODE_AUDIT, true>, resident_grid(k_colour<MODE_AUDIT, true>, &g_col_tla, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, d, round, colours, s);
	else if(use_nl && d->nl_k > 0) launch_round(k_colour<MODE_FAST, true>, resident_grid(k_colour<MODE_FAST, true>, &g_col_tl, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, d, round, colours, s);
	else if(aud) launch_round(k_colour<MODE_AUDIT, false>, resident_grid(k_colour<MODE_AUDIT, false>, &g_col_audit, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, d, round, colours, s);
	else launch_round(k_colour<MODE_FAST, false>, resident_grid(k_colour<MODE_FAST, false>, &g_col_fast, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, d, round, colours, s);
	*nl += 8;
	return (int) cudaGetLastError();
}

static void launch_energy(const ppi_dev *d, int mode, int use_nl, cudaStream_t s, long long *nl) {

	const int audit = d->audit_any;
	if(mode == PPI_EN_PARTNERS) { /* one lane per particle: the partner list is written in order */
		if(audit) k_energy<MODE_AUDIT, 1><<<resident_grid(k_energy<MODE_AUDIT, 1>, &g_a1), 128, 0, s>>>(*d, mode);
		else k_energy<MODE_FAST, 1><<<resident_grid(k_energy<MODE_FAST, 1>, &g_f1), 128, 0, s>>>(*d, mode);
	}
	else if(audit) k_energy<MODE_AUDIT, 4><<<resident_grid(k_energy<MODE_AUDIT, 4>, &g_a4), 128, 0, s>>>(*d, mode);
	else if(mode == PPI_EN_VOLUME && use_nl && d->nl_k > 0 && d->vpairs) { /* k_vol_plan cleared the queue */
		launch_pdl(k_energy_vol_pairs, resident_grid(k_energy_vol_pairs, &g_vol_pairs, VP_B), VP_B, s, *d);
		launch_pdl(k_vol_unsure, 4 * ppi_sm_count(), 128, s, *d); /* a warp per guard-band pair, on every SM's FP64 pipe */
		*nl += 1;
	}
	else if(mode == PPI_EN_VOLUME && use_nl && d->nl_k > 0)
		k_energy_vol<true><<<resident_grid(k_energy_vol<true>, &g_vol_list, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, s>>>(*d);
	else if(mode == PPI_EN_VOLUME) k_energy_vol<false><<<resident_grid(k_energy_vol<false>, &g_vol_grid, 32 * TILE_WARPS), 32 * TILE_WARPS, 0, s>>>(*d);
	else if(lanes_of(d) == 8) k_energy<MODE_FAST, 8><<<resident_grid(k_energy<MODE_FAST, 8>, &g_f8), 128, 0, s>>>(*d, mode);
	else k_energy<MODE_FAST, 4><<<resident_grid(k_energy<MODE_FAST, 4>, &g_f4), 128, 0, s>>>(*d, mode);
	*nl += 1;
}

extern "C" int ppi_energy(const ppi_dev *d, int mode, cudaStream_t s, long long *nl) {
	if(mode != PPI_EN_VOLUME) {
		k_energy_reset<<<(d->nrep + 63) / 64, 64, 0, s>>>(*d);
		*nl += 1;
	}
	launch_energy(d, mode, 0, s, nl);
	return (int) cudaGetLastError();
}

extern "C" int ppi_volume(const ppi_dev *d, long long sweep, int use_nl, cudaStream_t s, long long *nl) {
	/* the chain plan -> candidate-box energy -> guard band -> decide -> rescale, each launch overlapping its
	 * predecessor's tail (programmatic dependent launch; every kernel waits before its first access) */
	launch_pdl(k_vol_plan, (d->nrep + 63) / 64, 64, s, *d, sweep);
	launch_energy(d, PPI_EN_VOLUME, use_nl, s, nl);
	launch_pdl(k_vol_decide, (d->nrep + 63) / 64, 64, s, *d, sweep);
	if(d->ntot > 0) { /* one resident wave that loops: when no box is accepted (the usual case) it only reads a flag */
		const int nb = (d->ntot + 255) / 256, cap = 8 * ppi_sm_count();
		launch_pdl(k_vol_apply, nb < cap ? nb : cap, 256, s, *d);
	}
	*nl += 3;
	return (int) cudaGetLastError();
}

extern "C" int ppi_gram_schmidt(const ppi_dev *d, int first, int count, cudaStream_t s, long long *nl) {
	if(count <= 0) return 0;
	k_gram_schmidt<<<(count + 255) / 256, 256, 0, s>>>(*d, first, count);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_exchange(const ppi_dev *d, long long step, int attempts, cudaStream_t s, long long *nl) {
	if(attempts <= 0) return 0;
	k_exchange<<<d->nrep, EXCH_B, 0, s>>>(*d, step, attempts);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_reorder(const ppi_dev *d, cudaStream_t s, long long *nl) {
	if(d->ntot <= 0) return 0;
	k_gather<<<(d->ntot + 255) / 256, 256, 0, s>>>(*d);
	*nl += 1;
	cudaMemcpyAsync(d->rec, d->tmp_rec, sizeof(double) * PPI_REC * (size_t) d->ntot, cudaMemcpyDeviceToDevice, s);
	cudaMemcpyAsync(d->id, d->tmp_id, sizeof(int) * (size_t) d->ntot, cudaMemcpyDeviceToDevice, s);
	return (int) cudaGetLastError();
}

__global__ void k_set_counters(ppi_ctr *c, long long round, long long epoch, long long sweep) {
	c->round = round;
	c->epoch = epoch;
	c->sweep = sweep;
}

extern "C" int ppi_set_counters(const ppi_dev *d, long long round, long long epoch, long long sweep, cudaStream_t s, long long *nl) {
	k_set_counters<<<1, 1, 0, s>>>(d->ctr, round, epoch, sweep);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_canon(const ppi_dev *d, cudaStream_t s, long long *nl) {
	if(d->ntot <= 0) return 0;
	k_canon<<<(d->ntot + 255) / 256, 256, 0, s>>>(*d);
	*nl += 1;
	return (int) cudaGetLastError();
}

/* one wave of resident CTAs of a learned-move kernel (one warp each; dynamic shared memory: the
 * network's tile; tensor memory: MLP_WARP_TMEM_COLS columns per CTA of the SM's 512) */
template <typename F>
static int learned_grid(F f, int *cache) {
	if(*cache == 0) {
		if(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) LEARN_SMEM) != cudaSuccess) return -1;
		int nb = 0;
		if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, 32, LEARN_SMEM) != cudaSuccess || nb <= 1) {
			/* the shared-memory bound from the device limits (a grid beyond residency only queues) */
			int dev = 0, smem_sm = 0;
			cudaGetLastError();
			cudaGetDevice(&dev);
			cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
			nb = smem_sm / (int) (LEARN_SMEM + 1024);
			if(nb < 1) nb = 1;
		}
		if(nb > 512 / MLP_WARP_TMEM_COLS) nb = 512 / MLP_WARP_TMEM_COLS;
		*cache = nb * ppi_sm_count();
	}
	return *cache;
}

extern "C" int ppi_prepare(const ppi_dev *d) {
	(void) d;
	resident_grid(k_colour<MODE_AUDIT, false>, &g_col_audit, 32 * TILE_WARPS);
	resident_grid(k_colour<MODE_FAST, false>, &g_col_fast, 32 * TILE_WARPS);
	resident_grid(k_colour<MODE_AUDIT, true>, &g_col_tla, 32 * TILE_WARPS);
	resident_grid(k_colour<MODE_FAST, true>, &g_col_tl, 32 * TILE_WARPS);
	resident_grid(k_energy_vol<false>, &g_vol_grid, 32 * TILE_WARPS);
	resident_grid(k_energy_vol<true>, &g_vol_list, 32 * TILE_WARPS);
	resident_grid(k_energy_vol_pairs, &g_vol_pairs, VP_B);
	resident_grid(k_energy<MODE_AUDIT, 1>, &g_a1);
	resident_grid(k_energy<MODE_AUDIT, 4>, &g_a4);
	resident_grid(k_energy<MODE_FAST, 1>, &g_f1);
	resident_grid(k_energy<MODE_FAST, 4>, &g_f4);
	resident_grid(k_energy<MODE_FAST, 8>, &g_f8);
	round_grid();
	if(learned_grid(k_colour_learned<MODE_AUDIT>, &g_learn_audit) < 0 || learned_grid(k_colour_learned<MODE_FAST>, &g_learn_fast) < 0) return (int) cudaGetLastError();
	return (int) cudaGetLastError();
}

extern "C" int ppi_round_learned(const ppi_dev *d, long long round, const int *colours, int audit, cudaStream_t s, long long *nl) {
	if(audit || d->audit_any) {
		const int grid = learned_grid(k_colour_learned<MODE_AUDIT>, &g_learn_audit);
		if(grid < 0) return (int) cudaGetLastError();
		launch_round(k_colour_learned<MODE_AUDIT>, grid, 32, LEARN_SMEM, d, round, colours, s);
	}
	else {
		const int grid = learned_grid(k_colour_learned<MODE_FAST>, &g_learn_fast);
		if(grid < 0) return (int) cudaGetLastError();
		launch_round(k_colour_learned<MODE_FAST>, grid, 32, LEARN_SMEM, d, round, colours, s);
	}
	*nl += 8;
	return (int) cudaGetLastError();
}

extern "C" int ppi_learn_features(const ppi_dev *d, cudaStream_t s, long long *nl) {
	if(d->ntot <= 0) return 0;
	k_learn_features<<<(d->ntot + 127) / 128, 128, 0, s>>>(*d);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_learn_collect(const ppi_dev *d, long long snap, int col, int base, int count, cudaStream_t s, long long *nl) {
	if(count <= 0) return 0;
	if(d->audit_any) k_learn_collect<MODE_AUDIT><<<(count + 127) / 128, 128, 0, s>>>(*d, snap, col, base, count);
	else k_learn_collect<MODE_FAST><<<(count + 127) / 128, 128, 0, s>>>(*d, snap, col, base, count);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_export(const ppi_dev *d, int first, int count, cudaStream_t s, long long *nl) {
	if(count <= 0) return 0;
	k_export<<<(count + 255) / 256, 256, 0, s>>>(*d, first, count);
	*nl += 1;
	return (int) cudaGetLastError();
}

/* ------------------------------------------------------------------------------------------------ */
/* allocation-free energy of one configuration (pp_gpu_energy_noalloc)                               */
/*                                                                                                  */
/* For callers that may not allocate device memory: every scratch buffer of the energy pass (cell     */
/* grid, counting sort, FP32 working records, FP64 records) is carved out of one file-scope device    */
/* array of fixed size, so a call allocates nothing. The kernels are the engine's own (k_grid ...    */
/* k_energy), given a ppi_dev view whose pointers lie inside the array.                               */
/* ------------------------------------------------------------------------------------------------ */
#define NOALLOC_N 32768      /* particles */
#define NOALLOC_CELLS 131072 /* cells of the grid (even count >= 4 per axis, edge >= r_cut) */
#define NA_ALIGN(x) ((((size_t) (x)) + 255) & ~(size_t) 255)
#define NA_REC ((size_t) 0)
#define NA_STAGE (NA_REC + NA_ALIGN((size_t) NOALLOC_N * PPI_REC * sizeof(double)))
#define NA_SPOS (NA_STAGE + NA_ALIGN((size_t) NOALLOC_N * sizeof(float4)))
#define NA_SORI (NA_SPOS + NA_ALIGN((size_t) NOALLOC_N * sizeof(float4)))
#define NA_ID (NA_SORI + NA_ALIGN((size_t) NOALLOC_N * 3 * sizeof(float4)))
#define NA_REP (NA_ID + NA_ALIGN((size_t) NOALLOC_N * sizeof(int)))
#define NA_CELLOF (NA_REP + NA_ALIGN((size_t) NOALLOC_N * sizeof(int)))
#define NA_BONDS (NA_CELLOF + NA_ALIGN((size_t) NOALLOC_N * sizeof(int)))
#define NA_OVER (NA_BONDS + NA_ALIGN((size_t) NOALLOC_N * sizeof(int)))
#define NA_CCOUNT (NA_OVER + NA_ALIGN((size_t) NOALLOC_N * sizeof(int)))
#define NA_CSTART (NA_CCOUNT + NA_ALIGN((size_t) NOALLOC_CELLS * sizeof(int)))
#define NA_CCURSOR (NA_CSTART + NA_ALIGN((size_t) (NOALLOC_CELLS + 1) * sizeof(int)))
#define NA_CREP (NA_CCURSOR + NA_ALIGN((size_t) NOALLOC_CELLS * sizeof(int)))
#define NA_AUX (NA_CREP + NA_ALIGN((size_t) NOALLOC_CELLS * sizeof(int)))
#define NA_CLIST (NA_AUX + NA_ALIGN((size_t) (NOALLOC_CELLS / 1024 + 2) * sizeof(int)))
#define NA_COLCOUNT (NA_CLIST + NA_ALIGN((size_t) 8 * (NOALLOC_CELLS / 8 + 8) * sizeof(int4)))
#define NA_EFLAG (NA_COLCOUNT + NA_ALIGN(8 * sizeof(int)))
#define NA_RP (NA_EFLAG + NA_ALIGN((size_t) NOALLOC_N))
#define NA_RS (NA_RP + NA_ALIGN(sizeof(ppi_rparams)))
#define NA_GRID (NA_RS + NA_ALIGN(sizeof(ppi_rstate)))
#define NA_TOTAL (NA_GRID + NA_ALIGN(sizeof(ppi_grid)))

/* The scratch. Host code must not use its name as an address: the device address comes from
 * cudaGetSymbolAddress, looked up on every call with the caller's device and context current (an address
 * kept from an earlier call could belong to a context that a cudaDeviceReset has since destroyed). */
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

__global__ void k_noalloc_pack(ppi_dev d, const double *r, const double *R) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= d.ntot) return;
	double *o = d.rec + (size_t) i * PPI_REC;
	o[0] = r[3 * (size_t) i];
	o[1] = r[3 * (size_t) i + 1];
	o[2] = r[3 * (size_t) i + 2];
	o[PPI_Q] = 1.0;
	o[PPI_Q + 1] = 0.0;
	o[PPI_Q + 2] = 0.0;
	o[PPI_Q + 3] = 0.0;
	for(int k = 0; k < 9; k++) o[PPI_R0 + k] = R[9 * (size_t) i + k];
	d.id[i] = i;
	d.rep[i] = 0;
}

static int na_fail(char *err, int err_len, int code, const char *msg, const char *detail) {
	if(err && err_len > 0) snprintf(err, err_len, "%s%s%s", msg, detail ? ": " : "", detail ? detail : "");
	return code;
}

extern "C" int pp_gpu_energy_noalloc(int N, const double *r_dev, const double *R_dev, const double box[3], double kf_delta, double kf_cosmax,
		int *n_bonds_dev, int *n_overlaps_dev, double *E, int *overlap, char *err, int err_len) {
	if(err && err_len > 0) err[0] = '\0';
	if(box == NULL || E == NULL || overlap == NULL || N < 0 || (N > 0 && (r_dev == NULL || R_dev == NULL)))
		return na_fail(err, err_len, PP_ERR_ARG, "invalid arguments", NULL);
	if(!(kf_delta > 0. && kf_delta < 1.) || !(kf_cosmax > -1. && kf_cosmax < 1.)) return na_fail(err, err_len, PP_ERR_ARG, "KF_delta or KF_cosmax out of range", NULL);
	if(N > NOALLOC_N) {
		char b[96];
		snprintf(b, sizeof(b), "N = %d exceeds the static capacity of %d particles", N, NOALLOC_N);
		return na_fail(err, err_len, PP_ERR_CAPACITY, "pp_gpu_energy_noalloc", b);
	}
	ppi_rparams rp;
	ppi_model_params(N, kf_delta, kf_cosmax, &rp);
	long long cells = 1;
	for(int a = 0; a < 3; a++) {
		if(!(box[a] > 0.)) return na_fail(err, err_len, PP_ERR_ARG, "box sides must be positive", NULL);
		int n = (int) floor(box[a] / rp.w_min);
		if(n > PPI_MAX_AXIS_CELLS) n = PPI_MAX_AXIS_CELLS;
		n &= ~1;
		if(n < 4) return na_fail(err, err_len, PP_ERR_CAPACITY, "pp_gpu_energy_noalloc", "a box side is shorter than 4 cells of edge 1 + KF_delta");
		cells *= n;
	}
	if(cells > NOALLOC_CELLS) {
		char b[96];
		snprintf(b, sizeof(b), "the box needs %lld cells, the static capacity is %d", cells, NOALLOC_CELLS);
		return na_fail(err, err_len, PP_ERR_CAPACITY, "pp_gpu_energy_noalloc", b);
	}
	rp.cell_base = 0;
	rp.cell_cap = (int) cells;
	rp.p0 = 0;
	/* device address of the scratch in the current device's current context, looked up on every call
	 * (a table lookup once the module is loaded; the first call on a device loads it) */
	void *sym = NULL;
	cudaError_t c = cudaGetSymbolAddress(&sym, g_noalloc_scratch);
	if(c != cudaSuccess || sym == NULL) return na_fail(err, err_len, PP_ERR_CUDA, "cudaGetSymbolAddress", cudaGetErrorString(c));
	unsigned char *base = (unsigned char *) sym;
	ppi_dev d;
	memset(&d, 0, sizeof(d));
	d.nrep = 1;
	d.ntot = N;
	d.total_cells = (int) cells;
	d.clist_cap = (int) (cells / 8 + 8);
	d.rec = (double *) (base + NA_REC);
	d.tmp_rec = (double *) (base + NA_STAGE); /* float4 staging of the cell assignment */
	d.spos = (float4 *) (base + NA_SPOS);
	d.sori = (float4 *) (base + NA_SORI);
	d.id = (int *) (base + NA_ID);
	d.rep = (int *) (base + NA_REP);
	d.cellof = (int *) (base + NA_CELLOF);
	d.out_bonds = n_bonds_dev ? n_bonds_dev : (int *) (base + NA_BONDS);
	d.out_overlaps = n_overlaps_dev ? n_overlaps_dev : (int *) (base + NA_OVER);
	d.cell_count = (int *) (base + NA_CCOUNT);
	d.cell_start = (int *) (base + NA_CSTART);
	d.cell_part = (int *) (base + NA_CCURSOR);
	d.cell_rep = (int *) (base + NA_CREP);
	d.scan_aux = (int *) (base + NA_AUX);
	d.clist = (int4 *) (base + NA_CLIST);
	d.ccount = (int *) (base + NA_COLCOUNT);
	d.eflag = (unsigned char *) (base + NA_EFLAG);
	d.audit_any = 0;
	d.lanes = 0;
	d.rp = (ppi_rparams *) (base + NA_RP);
	d.rs = (ppi_rstate *) (base + NA_RS);
	d.grid = (ppi_grid *) (base + NA_GRID);
	/* the array keeps the previous call's contents: everything this call reads is written first */
	ppi_rstate rs;
	memset(&rs, 0, sizeof(rs));
	for(int a = 0; a < 3; a++) rs.box[a] = box[a];
	rs.V = box[0] * box[1] * box[2];
	if((c = cudaMemcpy(d.rp, &rp, sizeof(rp), cudaMemcpyHostToDevice)) != cudaSuccess ||
			(c = cudaMemcpy(d.rs, &rs, sizeof(rs), cudaMemcpyHostToDevice)) != cudaSuccess ||
			(c = cudaMemset(d.grid, 0, sizeof(ppi_grid))) != cudaSuccess || (c = cudaMemset(d.cell_rep, 0, sizeof(int) * (size_t) cells)) != cudaSuccess ||
			(c = cudaMemset(d.eflag, 0, (size_t) (N > 0 ? N : 1))) != cudaSuccess)
		return na_fail(err, err_len, PP_ERR_CUDA, "scratch set-up", cudaGetErrorString(c));
	long long nl = 0;
	if(N > 0) k_noalloc_pack<<<(N + 255) / 256, 256>>>(d, r_dev, R_dev);
	int rc = ppi_resort(&d, 0, 0, &nl);
	if(rc == 0) rc = ppi_energy(&d, PPI_EN_BONDS, 0, &nl);
	if(rc != 0) return na_fail(err, err_len, PP_ERR_CUDA, "kernel launch", cudaGetErrorString((cudaError_t) rc));
	if((c = cudaMemcpy(&rs, d.rs, sizeof(rs), cudaMemcpyDeviceToHost)) != cudaSuccess) return na_fail(err, err_len, PP_ERR_CUDA, "result copy", cudaGetErrorString(c));
	if(rs.error) return na_fail(err, err_len, PP_ERR_CAPACITY, "pp_gpu_energy_noalloc", "cell grid error on the device");
	*E = -0.5 * (double) rs.vol_bonds;
	*overlap = rs.vol_overlap;
	return PP_OK;
}
