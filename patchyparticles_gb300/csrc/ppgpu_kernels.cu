/*
 * ppgpu_kernels.cu -- sm_103a kernels of the roto-translation Monte Carlo engine (global checkerboard).
 *
 * Every `resort_every` rounds each replica gets a new cell grid (even number of cells per axis, edge >=
 * r_cut, random origin shift) and the particles are counting-sorted into cell order as 64-B FP32 working
 * records rebuilt from the FP64 canonical state:
 *   k_grid, k_assign, k_scan_*, k_scatter, k_cellfin (deterministic in-cell order, colour lists)
 * One round = the 8 colours of the 2x2x2 checkerboard, one launch each (k_colour): every non-empty
 * cell of the colour is one thread that performs one roto-translation attempt on a uniformly chosen
 * particle of the cell (MC_move_rototranslate, MC.c:311-340). Same-colour cells are never adjacent and a
 * move that leaves its cell is rejected, so concurrent moves never interact and the cell lists stay
 * valid for the whole epoch. The pair test is FP32 with an FP64 re-evaluation inside the guard band,
 * bit-identical to MC_would_interact (MC.c:232-266). Accepted moves update the FP64 state with FP64
 * arithmetic and the FP32 record in place.
 * k_energy: energy from scratch (per-particle bonds/overlaps, output.c:213-268) or of the NPT candidate
 * box (MC.c:487-495); k_vol_*: the NPT volume move (MC.c:450-513).
 */
#include "ppgpu.h"
#include "ppgpu_internal.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
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

__device__ __forceinline__ float u01(uint32_t v) { return (float) (v >> 8) * 0x1p-24f; } /* [0, 1) */
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) { return (double) (((uint64_t) a << 21) | (b >> 11)) * 0x1p-53; }

/* ------------------------------------------------------------------------------------------------ */
/* Reference-exact FP64 pair test: MC_would_interact (MC.c:232-266) with the patches of              */
/* MATRIX_VECTOR_MULTIPLICATION (utils.h:18-22). Every operation is an explicitly rounded IEEE        */
/* operation, so nothing is contracted into an FMA and the result equals the reference's bit for bit. */
/* ------------------------------------------------------------------------------------------------ */
__device__ __forceinline__ void patches64(const double *R, const double (*b)[3], double *P) {
#pragma unroll
	for(int i = 0; i < 4; i++) {
#pragma unroll
		for(int k = 0; k < 3; k++)
			P[3 * i + k] = __dadd_rn(__dadd_rn(__dmul_rn(R[3 * k + 0], b[i][0]), __dmul_rn(R[3 * k + 1], b[i][1])), __dmul_rn(R[3 * k + 2], b[i][2]));
	}
}

__device__ __forceinline__ double scalar64(const double *a, const double *b) {
	return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

/* returns -1 overlap, 0 no bond, 1 bond; optional diagnostics (dist2, max p cosine, max q cosine) */
__device__ int interact64(const double *rp, const double *Pp, const double *rq, const double *Pq, const double *box, double sqr_rcut, double cosmax,
		double *o_dist2, double *o_pmax, double *o_qmax) {
	double d[3];
#pragma unroll
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
		double pmax = -2., qmax = -2.;
		int pok = 0;
		for(int a = 0; a < 4; a++) {
			double pc = scalar64(d, Pp + 3 * a);
			pmax = fmax(pmax, pc);
			if(pc > cosmax) pok = 1;
		}
		for(int b = 0; b < 4; b++) {
			double qc = -scalar64(d, Pq + 3 * b);
			qmax = fmax(qmax, qc);
			if(pok && qc > cosmax) res = 1;
		}
		if(o_pmax) *o_pmax = pmax;
		if(o_qmax) *o_qmax = qmax;
	}
	return res;
}

/* candidate FP64 state of a move: r + disp, R . Q with Q the rotation of the quaternion (w, x, y, z)
 * given in FP32 and normalised in FP64. This is the engine's definition of the proposed state;
 * FP32 tests approximate it, FP64 re-evaluations and the accepted update use exactly these bits. */
__device__ __forceinline__ void candidate64(const double *rec, float4 q, float3 disp, double *r, double *R) {
	double w = q.x, x = q.y, y = q.z, z = q.w;
	double n = w * w + x * x + y * y + z * z;
	double inv = (double) (1.0f / (float) n);
	inv = inv * (2.0 - n * inv);
	inv = inv * (2.0 - n * inv);
	double s = 2.0 * inv;
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
	for(int k = 0; k < 3; k++) {
#pragma unroll
		for(int j = 0; j < 3; j++) {
			double acc = rec[3 + 3 * k + 0] * Q[0 + j];
			acc = fma(rec[3 + 3 * k + 1], Q[3 + j], acc);
			acc = fma(rec[3 + 3 * k + 2], Q[6 + j], acc);
			R[3 * k + j] = acc;
		}
	}
	r[0] = rec[0] + (double) disp.x;
	r[1] = rec[1] + (double) disp.y;
	r[2] = rec[2] + (double) disp.z;
}

/* Exact re-evaluation of one pair. p is the probing particle: kind 0 = its stored state, kind 1 = the
 * candidate of the current move (q, disp). vol_dir >= 0 scales coordinate vol_dir of both positions by
 * vol_f and uses box[vol_dir] = vol_side (the NPT candidate box, MC.c:471-478). */
__device__ __noinline__ int exact_pair(const double *__restrict__ rec_all, const ppi_rparams *rp, const double *box_in, int ps, int kind, float4 q,
		float3 disp, int qs, int vol_dir, double vol_f, double vol_side, double *o_dist2, double *o_pmax, double *o_qmax) {
	double rp_[3], Rp[9], rq[3], Pp[12], Pq[12], box[3];
	const double *recp = rec_all + (size_t) ps * PPI_REC;
	const double *recq = rec_all + (size_t) qs * PPI_REC;
	if(kind == 1) candidate64(recp, q, disp, rp_, Rp);
	else {
		for(int k = 0; k < 3; k++) rp_[k] = recp[k];
		for(int k = 0; k < 9; k++) Rp[k] = recp[3 + k];
	}
	for(int k = 0; k < 3; k++) {
		rq[k] = recq[k];
		box[k] = box_in[k];
	}
	if(vol_dir >= 0) {
		rp_[vol_dir] = __dmul_rn(rp_[vol_dir], vol_f);
		rq[vol_dir] = __dmul_rn(rq[vol_dir], vol_f);
		box[vol_dir] = vol_side;
	}
	patches64(Rp, rp->base, Pp);
	patches64(recq + 3, rp->base, Pq);
	return interact64(rp_, Pp, rq, Pq, box, rp->sqr_rcut, rp->cosmax, o_dist2, o_pmax, o_qmax);
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

__device__ __forceinline__ void atomicMaxFloatBits(unsigned int *addr, float v) {
	if(v > 0.f) atomicMax(addr, __float_as_uint(v)); /* positive floats order like their bit patterns */
}

/* audit: compare an FP32 decision with the exact one */
__device__ __noinline__ void audit_pair(const double *rec_all, const ppi_rparams *rp, ppi_rstate *rs, const double *box, int ps, int kind, float4 q,
		float3 disp, int qs, int vol_dir, double vol_f, double vol_side, int cl, PairF f) {
	double d2, pm = -2., qm = -2.;
	int ex = exact_pair(rec_all, rp, box, ps, kind, q, disp, qs, vol_dir, vol_f, vol_side, &d2, &pm, &qm);
	int exc = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
	if(cl != CL_UNSURE && cl != exc) atomicAdd(&rs->mismatches, 1ull);
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

__global__ void k_grid(ppi_dev d, long long epoch) {
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	ppi_grid *g = d.grid + r;
	U4 u = rng(rp, epoch, r, TAG_GRID, 0, 0);
	float us[3] = { u01(u.x), u01(u.y), u01(u.z) };
	int n[3];
	for(int a = 0; a < 3; a++) {
		int k = (int) floor(rs->box[a] / rp.w_min);
		if(k > PPI_MAX_AXIS_CELLS) k = PPI_MAX_AXIS_CELLS;
		k &= ~1; /* even: the 2x2x2 checkerboard needs alternating colours across the periodic boundary */
		if(k < 4) {
			rs->error = PPI_E_GRID;
			k = 4;
		}
		n[a] = k;
	}
	/* stay inside the reserved cell capacity by coarsening the longest axis (coarser cells stay valid) */
	while((long long) n[0] * n[1] * n[2] > rp.cell_cap) {
		int a = (n[0] >= n[1] && n[0] >= n[2]) ? 0 : (n[1] >= n[2] ? 1 : 2);
		if(n[a] <= 4) {
			rs->error = PPI_E_GRID;
			break;
		}
		n[a] -= 2;
	}
	for(int a = 0; a < 3; a++) {
		double w = rs->box[a] / n[a];
		g->n[a] = n[a];
		g->w[a] = w;
		g->wf[a] = (float) w;
		g->shift[a] = (double) us[a] * w;
		g->inv_w[a] = 1.0 / w;
		g->inv_L[a] = 1.0 / rs->box[a];
	}
	g->ncells = n[0] * n[1] * n[2];
}

/* cell of a slot in the current grid (FP64) and its cell-local coordinates (rounded to FP32) */
__global__ void k_assign(ppi_dev d, float4 *tmp) {
	int s = blockIdx.x * blockDim.x + threadIdx.x;
	if(s >= d.ntot) return;
	int r = d.rep[s];
	const ppi_grid g = d.grid[r];
	const double *x = d.rec + (size_t) s * PPI_REC;
	int c[3];
	float l[3];
	for(int a = 0; a < 3; a++) {
		double L = d.rs[r].box[a];
		double xw = x[a] - L * floor(x[a] * g.inv_L[a]);
		if(xw >= L) xw -= L; /* the reciprocal may round floor() one step off */
		else if(xw < 0.) xw += L;
		double u = (xw - g.shift[a]) * g.inv_w[a];
		int ci;
		double lo;
		if(u < 0.) {
			ci = g.n[a] - 1; /* below the shifted origin: the last cell, across the periodic boundary */
			lo = (xw + L) - (g.shift[a] + ci * g.w[a]);
		}
		else {
			ci = (int) floor(u);
			if(ci > g.n[a] - 1) ci = g.n[a] - 1;
			lo = xw - (g.shift[a] + ci * g.w[a]);
		}
		c[a] = ci;
		l[a] = (float) lo;
	}
	int gc = d.rp[r].cell_base + (c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
	d.cellof[s] = gc;
	tmp[s] = make_float4(l[0], l[1], l[2], __int_as_float(gc));
	atomicAdd(d.cell_count + gc, 1);
}

#define SCAN_B 1024
__global__ void k_scan_local(const int *in, int *out, int *cursor, int *aux, int n) {
	__shared__ int s[SCAN_B];
	int i = blockIdx.x * SCAN_B + threadIdx.x;
	int v = (i < n) ? in[i] : 0;
	s[threadIdx.x] = v;
	__syncthreads();
	for(int off = 1; off < SCAN_B; off <<= 1) {
		int t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
		__syncthreads();
		s[threadIdx.x] += t;
		__syncthreads();
	}
	if(i < n) {
		out[i] = s[threadIdx.x] - v;
		cursor[i] = 0;
	}
	if(threadIdx.x == SCAN_B - 1) aux[blockIdx.x] = s[SCAN_B - 1];
}

__global__ void k_scan_top(int *aux, int nblocks, int *total_out) {
	__shared__ int s[SCAN_B];
	int carry = 0;
	for(int base = 0; base < nblocks; base += SCAN_B) {
		int i = base + threadIdx.x;
		int v = (i < nblocks) ? aux[i] : 0;
		s[threadIdx.x] = v;
		__syncthreads();
		for(int off = 1; off < SCAN_B; off <<= 1) {
			int t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
			__syncthreads();
			s[threadIdx.x] += t;
			__syncthreads();
		}
		if(i < nblocks) aux[i] = carry + s[threadIdx.x] - v;
		int tot = s[SCAN_B - 1];
		__syncthreads();
		carry += tot;
	}
	if(threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(int *out, const int *aux, int n) {
	int i = blockIdx.x * SCAN_B + threadIdx.x;
	if(i < n) out[i] += aux[blockIdx.x];
}

__global__ void k_scatter(ppi_dev d, const float4 *tmp) {
	int s = blockIdx.x * blockDim.x + threadIdx.x;
	if(s >= d.ntot) return;
	int gc = d.cellof[s];
	int pos = d.cell_start[gc] + atomicAdd(d.cell_cursor + gc, 1);
	const double *R = d.rec + (size_t) s * PPI_REC + 3;
	float4 a = tmp[s];
	a.w = __int_as_float(s);
	float4 *o = d.srec + 4 * (size_t) pos;
	o[0] = a;
	o[1] = make_float4((float) R[0], (float) R[3], (float) R[6], (float) R[1]); /* c0 = (R00, R10, R20), c1.x = R01 */
	o[2] = make_float4((float) R[4], (float) R[7], (float) R[2], (float) R[5]); /* c1.y, c1.z, c2.x = R02, c2.y = R12 */
	o[3] = make_float4((float) R[8], __int_as_float(d.id[s]), __int_as_float(gc), 0.f);
}

/* per cell: deterministic order (ascending particle id), and the colour lists of non-empty cells */
__global__ void k_cellfin(ppi_dev d) {
	int gc = blockIdx.x * blockDim.x + threadIdx.x;
	if(gc >= d.total_cells) return;
	int r = d.cell_rep[gc];
	const ppi_grid &g = d.grid[r];
	int local = gc - d.rp[r].cell_base;
	if(local >= g.ncells) return;
	int a = d.cell_start[gc], b = d.cell_start[gc + 1];
	if(b <= a) return;
	float4 *v = d.srec;
	for(int i = a + 1; i < b; i++) {
		float4 x0 = v[4 * i], x1 = v[4 * i + 1], x2 = v[4 * i + 2], x3 = v[4 * i + 3];
		int key = __float_as_int(x3.y);
		int j = i - 1;
		while(j >= a && __float_as_int(v[4 * j + 3].y) > key) {
			v[4 * (j + 1)] = v[4 * j];
			v[4 * (j + 1) + 1] = v[4 * j + 1];
			v[4 * (j + 1) + 2] = v[4 * j + 2];
			v[4 * (j + 1) + 3] = v[4 * j + 3];
			j--;
		}
		v[4 * (j + 1)] = x0;
		v[4 * (j + 1) + 1] = x1;
		v[4 * (j + 1) + 2] = x2;
		v[4 * (j + 1) + 3] = x3;
	}
	int cx = local % g.n[0], cy = (local / g.n[0]) % g.n[1], cz = local / (g.n[0] * g.n[1]);
	int col = (cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2);
	int idx = atomicAdd(d.ccount + col, 1);
	if(idx < d.clist_cap) d.clist[col * d.clist_cap + idx] = gc;
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

struct Probe {
	float4 po;      /* old cell-local position */
	float3 pn;      /* candidate cell-local position */
	float cpo[9], cpn[9];
	int i, pslot;
	float4 q;
	float3 disp;
};

/* tests candidate jq (smem-free: records read from the global cell-sorted array) against the old and new
 * state of the moving particle; returns 1 if the new state overlaps */
__device__ __forceinline__ int test_candidate(const ppi_dev &d, const ppi_rparams &rp, ppi_rstate *rs, const double *box, const Probe &P, int jq, float ox,
		float oy, float oz, float sqr_rcut, float cosmax, float basef, float eps, int &bo, int &bn, Acc &A) {
	float4 qa = d.srec[4 * (size_t) jq];
	float dxo = (qa.x - P.po.x) + ox, dyo = (qa.y - P.po.y) + oy, dzo = (qa.z - P.po.z) + oz;
	float dxn = (qa.x - P.pn.x) + ox, dyn = (qa.y - P.pn.y) + oy, dzn = (qa.z - P.pn.z) + oz;
	float r2o = fmaf(dxo, dxo, fmaf(dyo, dyo, dzo * dzo));
	float r2n = fmaf(dxn, dxn, fmaf(dyn, dyn, dzn * dzn));
	A.pairs += 2;
	int qslot = __float_as_int(qa.w);
	if(r2o >= sqr_rcut + eps && r2n >= sqr_rcut + eps) {
		if(rp.audit) {
			PairF f;
			f.pmax = f.qmax = -2.f;
			f.r2 = r2o;
			audit_pair(d.rec, &rp, rs, box, P.pslot, 0, P.q, P.disp, qslot, -1, 1., 0., CL_NONE, f);
			f.r2 = r2n;
			audit_pair(d.rec, &rp, rs, box, P.pslot, 1, P.q, P.disp, qslot, -1, 1., 0., CL_NONE, f);
		}
		return 0;
	}
	float4 qb = d.srec[4 * (size_t) jq + 1], qc = d.srec[4 * (size_t) jq + 2];
	float qd = d.srec[4 * (size_t) jq + 3].x;
	float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd };
	PairF fo, fn;
	int clo = classify(dxo, dyo, dzo, P.cpo, cq, sqr_rcut, cosmax, basef, eps, &fo);
	int cln = classify(dxn, dyn, dzn, P.cpn, cq, sqr_rcut, cosmax, basef, eps, &fn);
	if(rp.audit) {
		audit_pair(d.rec, &rp, rs, box, P.pslot, 0, P.q, P.disp, qslot, -1, 1., 0., clo, fo);
		audit_pair(d.rec, &rp, rs, box, P.pslot, 1, P.q, P.disp, qslot, -1, 1., 0., cln, fn);
	}
	if(clo == CL_UNSURE) {
		A.fallbacks++;
		int ex = exact_pair(d.rec, &rp, box, P.pslot, 0, P.q, P.disp, qslot, -1, 1., 0., nullptr, nullptr, nullptr);
		clo = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
	}
	if(cln == CL_UNSURE) {
		A.fallbacks++;
		int ex = exact_pair(d.rec, &rp, box, P.pslot, 1, P.q, P.disp, qslot, -1, 1., 0., nullptr, nullptr, nullptr);
		cln = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
	}
	bo += (clo == CL_BOND);
	bn += (cln == CL_BOND);
	return cln == CL_OVER;
}

/* accepted move: FP64 update of the canonical state (candidate64) and the FP32 working record */
__device__ __noinline__ void commit_move(const ppi_dev &d, int i, int pslot, float4 q, float3 disp, float3 pn, float pw, const float *cpn) {
	double *rec = d.rec + (size_t) pslot * PPI_REC;
	double old[PPI_REC], nr[3], nR[9];
#pragma unroll
	for(int k = 0; k < PPI_REC; k++) old[k] = rec[k];
	candidate64(old, q, disp, nr, nR);
	rec[0] = nr[0];
	rec[1] = nr[1];
	rec[2] = nr[2];
#pragma unroll
	for(int k = 0; k < 9; k++) rec[3 + k] = nR[k];
	float4 *o = d.srec + 4 * (size_t) i;
	o[0] = make_float4(pn.x, pn.y, pn.z, pw);
	o[1] = make_float4(cpn[0], cpn[1], cpn[2], cpn[3]);
	o[2] = make_float4(cpn[4], cpn[5], cpn[6], cpn[7]);
	o[3].x = cpn[8];
}

__device__ void attempt(const ppi_dev &d, int gc, long long round, Acc &A) {
	int r = d.cell_rep[gc];
	if(r != A.r) {
		flush_thread(d, A);
		A.r = r;
	}

	const ppi_rparams &rp = d.rp[r];
	const ppi_grid &g = d.grid[r];
	ppi_rstate *rs = d.rs + r;
	const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
	const int local = gc - rp.cell_base;
	const int cx = local % nx, cy = (local / nx) % ny, cz = local / (nx * ny);
	const int c0 = d.cell_start[gc], cnt = d.cell_start[gc + 1] - c0;
	U4 r1 = rng(rp, round, r, TAG_MOVE, (uint32_t) local, 0);
	U4 r2 = rng(rp, round, r, TAG_MOVE, (uint32_t) local, 1);
	Probe P;
	P.i = c0 + (int) __umulhi(r1.x, (uint32_t) cnt);
	A.tries++;
	P.disp = make_float3((u01(r1.y) - 0.5f) * rp.disp_max_f, (u01(r1.z) - 0.5f) * rp.disp_max_f, (u01(r1.w) - 0.5f) * rp.disp_max_f);
	const float wx = g.wf[0], wy = g.wf[1], wz = g.wf[2];
	P.po = d.srec[4 * (size_t) P.i];
	P.pn = make_float3(P.po.x + P.disp.x, P.po.y + P.disp.y, P.po.z + P.disp.z);
	/* a move that leaves the cell is rejected: cells stay valid and same-colour cells stay independent */
	if(!(P.pn.x >= 0.f && P.pn.x < wx && P.pn.y >= 0.f && P.pn.y < wy && P.pn.z >= 0.f && P.pn.z < wz)) return;
	/* rotation: angle uniform in [0, Theta_max), axis uniform on the sphere (inversion method) */
	float theta = u01(r2.x) * rp.theta_max_f;
	float zc = 1.f - 2.f * u01(r2.y);
	float phi = 6.283185307179586f * u01(r2.z);
	float sr = sqrtf(fmaxf(0.f, 1.f - zc * zc));
	float sp, cp, sh, ch;
	__sincosf(phi, &sp, &cp);
	__sincosf(0.5f * theta, &sh, &ch);
	P.q = make_float4(ch, sh * sr * cp, sh * sr * sp, sh * zc);
	{
		float4 b = d.srec[4 * (size_t) P.i + 1], c = d.srec[4 * (size_t) P.i + 2];
		float dd = d.srec[4 * (size_t) P.i + 3].x;
		P.cpo[0] = b.x;
		P.cpo[1] = b.y;
		P.cpo[2] = b.z;
		P.cpo[3] = b.w;
		P.cpo[4] = c.x;
		P.cpo[5] = c.y;
		P.cpo[6] = c.z;
		P.cpo[7] = c.w;
		P.cpo[8] = dd;
		float w = P.q.x, x = P.q.y, y = P.q.z, z = P.q.w;
		float Q[9];
		Q[0] = 1.f - 2.f * (y * y + z * z);
		Q[1] = 2.f * (x * y - w * z);
		Q[2] = 2.f * (x * z + w * y);
		Q[3] = 2.f * (x * y + w * z);
		Q[4] = 1.f - 2.f * (x * x + z * z);
		Q[5] = 2.f * (y * z - w * x);
		Q[6] = 2.f * (x * z - w * y);
		Q[7] = 2.f * (y * z + w * x);
		Q[8] = 1.f - 2.f * (x * x + y * y);
#pragma unroll
		for(int jj = 0; jj < 3; jj++)
#pragma unroll
			for(int k3 = 0; k3 < 3; k3++) P.cpn[3 * jj + k3] = fmaf(P.cpo[k3], Q[jj], fmaf(P.cpo[3 + k3], Q[3 + jj], P.cpo[6 + k3] * Q[6 + jj]));
	}
	P.pslot = __float_as_int(P.po.w);
	const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
	const float sqr_rcut = rp.sqr_rcut_f, cosmax = rp.cosmax_f, basef = rp.base_f;
	double box[3] = { rs->box[0], rs->box[1], rs->box[2] };
	const int *cs = d.cell_start;
	int bo = 0, bn = 0, over = 0;
	for(int rr = 0; rr < 9 && !over; rr++) {
		int dy = rr % 3 - 1, dz = rr / 3 - 1;
		int yy = cy + dy, zz = cz + dz;
		yy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
		zz = zz < 0 ? zz + nz : (zz >= nz ? zz - nz : zz);
		int rowbase = rp.cell_base + (zz * ny + yy) * nx;
		float oy = dy * wy, oz = dz * wz;
		if(cx >= 1 && cx <= nx - 2) {
			/* the three x-neighbours are consecutive cells: one contiguous range */
			int j0 = cs[rowbase + cx - 1], b1 = cs[rowbase + cx], b2 = cs[rowbase + cx + 1], j3 = cs[rowbase + cx + 2];
			for(int jq = j0; jq < j3; jq++) {
				if(jq == P.i) continue;
				float ox = jq < b1 ? -wx : (jq < b2 ? 0.f : wx);
				if(test_candidate(d, rp, rs, box, P, jq, ox, oy, oz, sqr_rcut, cosmax, basef, eps, bo, bn, A)) {
					over = 1;
					break;
				}
			}
		}
		else {
			for(int dx = -1; dx <= 1 && !over; dx++) {
				int xx = cx + dx;
				xx = xx < 0 ? xx + nx : (xx >= nx ? xx - nx : xx);
				int j0 = cs[rowbase + xx], j1 = cs[rowbase + xx + 1];
				float ox = dx * wx;
				for(int jq = j0; jq < j1; jq++) {
					if(jq == P.i) continue;
					if(test_candidate(d, rp, rs, box, P, jq, ox, oy, oz, sqr_rcut, cosmax, basef, eps, bo, bn, A)) {
						over = 1;
						break;
					}
				}
			}
		}
	}
	if(over) return;
	int dE = bo - bn; /* E = -bonds */
	if(dE > 0) {
		U4 r3 = rng(rp, round, r, TAG_MOVE, (uint32_t) local, 2);
		uint64_t U = ((uint64_t) r3.x << 21) | (r3.y >> 11);
		if(!(U < rp.acc_thr[dE < 31 ? dE : 31])) return;
	}
	A.acc++;
	A.dbonds += bn - bo;
	commit_move(d, P.i, P.pslot, P.q, P.disp, P.pn, P.po.w, P.cpn);
}

__global__ void __launch_bounds__(128) k_colour(ppi_dev d, long long round, int col) {
	int cnt = d.ccount[col];
	if(cnt > d.clist_cap) cnt = d.clist_cap;
	if(blockIdx.x * blockDim.x >= cnt) return; /* the whole CTA has no entry: leave before any reduction */
	Acc A;
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	int stride = gridDim.x * blockDim.x;
	for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += stride) attempt(d, d.clist[col * d.clist_cap + e], round, A);
	flush_block(d, A);
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

__global__ void __launch_bounds__(128) k_energy(ppi_dev d, int mode) {
	int stride = gridDim.x * blockDim.x;
	if(blockIdx.x * blockDim.x >= d.ntot) return;
	Acc A; /* A.tries = bonds counted, pairs, fallbacks */
	A.r = -1;
	A.tries = A.acc = A.pairs = A.fallbacks = 0;
	A.dbonds = 0;
	float4 qz = make_float4(1.f, 0.f, 0.f, 0.f);
	float3 dz0 = make_float3(0.f, 0.f, 0.f);
	for(int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.ntot; k += stride) {
		float4 pa = d.srec[4 * (size_t) k];
		float4 pb = d.srec[4 * (size_t) k + 1], pc = d.srec[4 * (size_t) k + 2], pd = d.srec[4 * (size_t) k + 3];
		int gc = __float_as_int(pd.z);
		int r = d.cell_rep[gc];
		if(r != A.r) {
			energy_flush_thread(d, A);
			A.r = r;
		}
		const ppi_rparams &rp = d.rp[r];
		const ppi_grid &g = d.grid[r];
		ppi_rstate *rs = d.rs + r;
		int sdir = -1;
		float sf = 1.f;
		double vf = 1.0, vside = 0.0;
		if(mode == PPI_EN_VOLUME) {
			if(g.vol_dir < 0 || rs->vol_overlap) continue;
			sdir = g.vol_dir;
			sf = g.vol_ff;
			vf = g.vol_f;
			vside = g.vol_side;
		}
		float w[3] = { g.wf[0], g.wf[1], g.wf[2] };
		float pl[3] = { pa.x, pa.y, pa.z };
		if(sdir >= 0) {
			w[sdir] *= sf;
			pl[sdir] *= sf;
		}
		float cp[9] = { pb.x, pb.y, pb.z, pb.w, pc.x, pc.y, pc.z, pc.w, pd.x };
		const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
		const int local = gc - rp.cell_base;
		const int cx = local % nx, cy = (local / nx) % ny, cz = local / (nx * ny);
		const float eps = rp.precision == 1 ? 1e30f : rp.eps_f;
		const float sqr_rcut = rp.sqr_rcut_f, cosmax = rp.cosmax_f, basef = rp.base_f;
		double box[3] = { rs->box[0], rs->box[1], rs->box[2] };
		int pslot = __float_as_int(pa.w);
		int nb = 0, no = 0;
		int *partners = (mode == PPI_EN_PARTNERS) ? d.out_partners + (size_t) pslot * PPI_MAX_PARTNERS : nullptr;
		for(int dz = -1; dz <= 1; dz++)
			for(int dy = -1; dy <= 1; dy++)
				for(int dx = -1; dx <= 1; dx++) {
					int xx = cx + dx, yy = cy + dy, zz = cz + dz;
					xx = xx < 0 ? xx + nx : (xx >= nx ? xx - nx : xx);
					yy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
					zz = zz < 0 ? zz + nz : (zz >= nz ? zz - nz : zz);
					int cell = rp.cell_base + (zz * ny + yy) * nx + xx;
					int j0 = d.cell_start[cell], j1 = d.cell_start[cell + 1];
					float ox = dx * w[0], oy = dy * w[1], oz = dz * w[2];
					for(int jq = j0; jq < j1; jq++) {
						if(jq == k) continue;
						float4 qa = d.srec[4 * (size_t) jq];
						float ql[3] = { qa.x, qa.y, qa.z };
						if(sdir >= 0) ql[sdir] *= sf;
						float ddx = (ql[0] - pl[0]) + ox, ddy = (ql[1] - pl[1]) + oy, ddz = (ql[2] - pl[2]) + oz;
						float r2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
						A.pairs++;
						int qslot = __float_as_int(qa.w);
						if(r2 >= sqr_rcut + eps) {
							if(rp.audit) {
								PairF f;
								f.r2 = r2;
								f.pmax = f.qmax = -2.f;
								audit_pair(d.rec, &rp, rs, box, pslot, 0, qz, dz0, qslot, sdir, vf, vside, CL_NONE, f);
							}
							continue;
						}
						float4 qb = d.srec[4 * (size_t) jq + 1], qc = d.srec[4 * (size_t) jq + 2];
						float qd = d.srec[4 * (size_t) jq + 3].x;
						float cq[9] = { qb.x, qb.y, qb.z, qb.w, qc.x, qc.y, qc.z, qc.w, qd };
						PairF f;
						int cl = classify(ddx, ddy, ddz, cp, cq, sqr_rcut, cosmax, basef, eps, &f);
						if(rp.audit) audit_pair(d.rec, &rp, rs, box, pslot, 0, qz, dz0, qslot, sdir, vf, vside, cl, f);
						if(cl == CL_UNSURE) {
							A.fallbacks++;
							int ex = exact_pair(d.rec, &rp, box, pslot, 0, qz, dz0, qslot, sdir, vf, vside, nullptr, nullptr, nullptr);
							cl = ex == -1 ? CL_OVER : (ex == 1 ? CL_BOND : CL_NONE);
						}
						if(cl == CL_BOND) {
							if(partners && nb < PPI_MAX_PARTNERS) partners[nb] = __float_as_int(d.srec[4 * (size_t) jq + 3].y);
							nb++;
						}
						no += (cl == CL_OVER);
					}
				}
		if(mode != PPI_EN_VOLUME) {
			d.out_bonds[pslot] = nb;
			d.out_overlaps[pslot] = no;
		}
		A.tries += nb;
		if(no && !rs->vol_overlap) atomicExch(&rs->vol_overlap, 1); /* visible at once: lets the others skip work */
	}
	energy_flush_block(d, A);
}

__global__ void k_energy_reset(ppi_dev d) {
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	d.rs[r].vol_bonds = 0;
	d.rs[r].vol_overlap = 0;
	d.rs[r].vol_accept = 0;
}

/* ------------------------------------------------------------------------------------------------ */
/* NPT volume move (MC.c:450-513)                                                                   */
/* ------------------------------------------------------------------------------------------------ */
__global__ void k_vol_plan(ppi_dev d, long long sweep) {
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	const ppi_rparams &rp = d.rp[r];
	ppi_rstate *rs = d.rs + r;
	ppi_grid *g = d.grid + r;
	rs->vol_bonds = 0;
	rs->vol_overlap = 0;
	rs->vol_accept = 0;
	g->vol_dir = -1;
	if(rp.ensemble != 5 || rp.N <= 0) return;
	U4 u = rng(rp, sweep, r, TAG_VOL, 0, 0);
	/* random axis, ln V' = ln V + (R - 0.5) rescale_factor_max, one side takes the whole change (MC.c:456-472) */
	int dir = (int) (u01d(u.x, u.y) * 3.0);
	if(dir > 2) dir = 2;
	double V0 = rs->box[0] * rs->box[1] * rs->box[2];
	double lnV = log(V0) + (u01d(u.z, u.w) - 0.5) * rp.rescale_max;
	double V1 = exp(lnV);
	double side = V1;
	for(int i = 0; i < 3; i++)
		if(i != dir) side /= rs->box[i];
	g->vol_dir = dir;
	g->vol_side = side;
	g->vol_f = side / rs->box[dir];
	g->vol_ff = (float) g->vol_f;
	g->vol_V0 = V0;
	g->vol_V1 = V1;
}

__global__ void k_vol_decide(ppi_dev d, long long sweep) {
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= d.nrep) return;
	const ppi_rparams &rp = d.rp[r];
	ppi_grid *g = d.grid + r;
	ppi_rstate *rs = d.rs + r;
	if(g->vol_dir < 0) return;
	rs->tries[6]++;
	long long nb_new = rs->vol_bonds / 2; /* every bonded pair was counted from both sides */
	double dE = (double) (rs->bonds - nb_new);
	double dV = g->vol_V1 - g->vol_V0;
	double arg = -(rp.P * dV + dE) / rp.T + (double) (rp.N + 1) * log(g->vol_f); /* MC.c:497-498 */
	U4 u = rng(rp, sweep, r, TAG_VOL, 0, 1);
	if(!rs->vol_overlap && u01d(u.x, u.y) < exp(arg)) {
		int a = g->vol_dir;
		rs->vol_accept = 1;
		rs->box[a] = g->vol_side;
		rs->V = g->vol_V1;
		rs->bonds = nb_new;
		rs->accepted[6]++;
		/* the cell grid scales with the box: cell membership is unchanged */
		g->w[a] *= g->vol_f;
		g->shift[a] *= g->vol_f;
		g->wf[a] = (float) g->w[a];
		g->inv_w[a] = 1.0 / g->w[a];
		g->inv_L[a] = 1.0 / rs->box[a];
	}
}

__global__ void k_vol_apply(ppi_dev d) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= d.ntot) return;
	/* canonical positions (slot k) */
	int r = d.rep[k];
	if(d.rs[r].vol_accept) {
		const ppi_grid &g = d.grid[r];
		double *rec = d.rec + (size_t) k * PPI_REC;
		rec[g.vol_dir] = __dmul_rn(rec[g.vol_dir], g.vol_f); /* p->r[dir] *= rescale_factor (MC.c:477) */
	}
	/* working record (sorted position k) */
	float4 *o = d.srec + 4 * (size_t) k;
	int gc = __float_as_int(o[3].z);
	int r2 = d.cell_rep[gc];
	if(d.rs[r2].vol_accept) {
		const ppi_grid &g = d.grid[r2];
		float4 a = o[0];
		if(g.vol_dir == 0) a.x *= g.vol_ff;
		else if(g.vol_dir == 1) a.y *= g.vol_ff;
		else a.z *= g.vol_ff;
		o[0] = a;
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* gram_schmidt, reorder                                                                            */
/* ------------------------------------------------------------------------------------------------ */
__device__ void normalize64(double *v) {
	double norm = __dsqrt_rn(scalar64(v, v));
	v[0] = __ddiv_rn(v[0], norm);
	v[1] = __ddiv_rn(v[1], norm);
	v[2] = __ddiv_rn(v[2], norm);
}

/* gram_schmidt (utils.c:91-113) on the orientation rows, with explicitly rounded operations */
__global__ void k_gram_schmidt(ppi_dev d, int first, int count) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= count) return;
	double *R = d.rec + (size_t) (first + k) * PPI_REC + 3;
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
		R[i] = v1[i];
		R[3 + i] = v2[i];
		R[6 + i] = v3[i];
	}
}

/* physical reorder of the canonical state into the current cell order (locality of the FP64 updates) */
__global__ void k_gather(ppi_dev d) {
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= d.ntot) return;
	float4 *o = d.srec + 4 * (size_t) k;
	int s = __float_as_int(o[0].w);
	const double *src = d.rec + (size_t) s * PPI_REC;
	double *dst = d.tmp_rec + (size_t) k * PPI_REC;
	for(int j = 0; j < PPI_REC; j++) dst[j] = src[j];
	d.tmp_id[k] = d.id[s];
	o[0].w = __int_as_float(k);
}

/* ------------------------------------------------------------------------------------------------ */
/* launchers                                                                                        */
/* ------------------------------------------------------------------------------------------------ */
static int g_sms = 0;

extern "C" int ppi_sm_count(void) {
	if(g_sms == 0) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
		if(g_sms <= 0) g_sms = 1;
	}
	return g_sms;
}

extern "C" int ppi_resort(const ppi_dev *d, long long epoch, cudaStream_t s, long long *nl) {
	float4 *tmp = (float4 *) d->tmp_rec; /* ntot float4 fit in the reorder scratch */
	cudaMemsetAsync(d->cell_count, 0, sizeof(int) * (size_t) d->total_cells, s);
	cudaMemsetAsync(d->ccount, 0, sizeof(int) * 8, s);
	k_grid<<<(d->nrep + 63) / 64, 64, 0, s>>>(*d, epoch);
	int nb = (d->ntot + 255) / 256;
	if(nb > 0) k_assign<<<nb, 256, 0, s>>>(*d, tmp);
	int sb = (d->total_cells + SCAN_B - 1) / SCAN_B;
	k_scan_local<<<sb, SCAN_B, 0, s>>>(d->cell_count, d->cell_start, d->cell_cursor, d->scan_aux, d->total_cells);
	k_scan_top<<<1, SCAN_B, 0, s>>>(d->scan_aux, sb, d->cell_start + d->total_cells);
	k_scan_add<<<sb, SCAN_B, 0, s>>>(d->cell_start, d->scan_aux, d->total_cells);
	if(nb > 0) k_scatter<<<nb, 256, 0, s>>>(*d, tmp);
	k_cellfin<<<(d->total_cells + 255) / 256, 256, 0, s>>>(*d);
	*nl += 5 + (nb > 0 ? 2 : 0);
	return (int) cudaGetLastError();
}

extern "C" int ppi_round(const ppi_dev *d, long long round, const int *colours, cudaStream_t s, long long *nl) {
	int grid = ppi_sm_count() * 8;
	for(int ci = 0; ci < 8; ci++) k_colour<<<grid, 128, 0, s>>>(*d, round, colours[ci]);
	*nl += 8;
	return (int) cudaGetLastError();
}

extern "C" int ppi_energy(const ppi_dev *d, int mode, cudaStream_t s, long long *nl) {
	if(mode != PPI_EN_VOLUME) {
		k_energy_reset<<<(d->nrep + 63) / 64, 64, 0, s>>>(*d);
		*nl += 1;
	}
	int grid = ppi_sm_count() * 8;
	k_energy<<<grid, 128, 0, s>>>(*d, mode);
	*nl += 1;
	return (int) cudaGetLastError();
}

extern "C" int ppi_volume(const ppi_dev *d, long long sweep, cudaStream_t s, long long *nl) {
	k_vol_plan<<<(d->nrep + 63) / 64, 64, 0, s>>>(*d, sweep);
	int grid = ppi_sm_count() * 8;
	k_energy<<<grid, 128, 0, s>>>(*d, PPI_EN_VOLUME);
	k_vol_decide<<<(d->nrep + 63) / 64, 64, 0, s>>>(*d, sweep);
	if(d->ntot > 0) k_vol_apply<<<(d->ntot + 255) / 256, 256, 0, s>>>(*d);
	*nl += 4;
	return (int) cudaGetLastError();
}

extern "C" int ppi_gram_schmidt(const ppi_dev *d, int first, int count, cudaStream_t s, long long *nl) {
	if(count <= 0) return 0;
	k_gram_schmidt<<<(count + 255) / 256, 256, 0, s>>>(*d, first, count);
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
#define NA_SREC (NA_STAGE + NA_ALIGN((size_t) NOALLOC_N * sizeof(float4)))
#define NA_ID (NA_SREC + NA_ALIGN((size_t) NOALLOC_N * 4 * sizeof(float4)))
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
#define NA_COLCOUNT (NA_CLIST + NA_ALIGN((size_t) 8 * (NOALLOC_CELLS / 8 + 8) * sizeof(int)))
#define NA_RP (NA_COLCOUNT + NA_ALIGN(8 * sizeof(int)))
#define NA_RS (NA_RP + NA_ALIGN(sizeof(ppi_rparams)))
#define NA_GRID (NA_RS + NA_ALIGN(sizeof(ppi_rstate)))
#define NA_TOTAL (NA_GRID + NA_ALIGN(sizeof(ppi_grid)))

/* The scratch. Host code must not use its name as an address: the device address comes from
 * cudaGetSymbolAddress (g_noalloc_base, once per device). */
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_TOTAL];

#define NOALLOC_MAX_DEVICES 64
static void *g_noalloc_base[NOALLOC_MAX_DEVICES];

__global__ void k_noalloc_pack(ppi_dev d, const double *r, const double *R) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= d.ntot) return;
	double *o = d.rec + (size_t) i * PPI_REC;
	o[0] = r[3 * (size_t) i];
	o[1] = r[3 * (size_t) i + 1];
	o[2] = r[3 * (size_t) i + 2];
	for(int k = 0; k < 9; k++) o[3 + k] = R[9 * (size_t) i + k];
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
	/* device address of the scratch, looked up once per device with that device current */
	int dev = 0;
	cudaError_t c = cudaGetDevice(&dev);
	if(c != cudaSuccess) return na_fail(err, err_len, PP_ERR_CUDA, "cudaGetDevice", cudaGetErrorString(c));
	if(dev < 0 || dev >= NOALLOC_MAX_DEVICES) return na_fail(err, err_len, PP_ERR_CUDA, "device ordinal out of range", NULL);
	if(g_noalloc_base[dev] == NULL) {
		void *p = NULL;
		c = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(c != cudaSuccess || p == NULL) return na_fail(err, err_len, PP_ERR_CUDA, "cudaGetSymbolAddress", cudaGetErrorString(c));
		g_noalloc_base[dev] = p;
	}
	unsigned char *base = (unsigned char *) g_noalloc_base[dev];
	ppi_dev d;
	memset(&d, 0, sizeof(d));
	d.nrep = 1;
	d.ntot = N;
	d.total_cells = (int) cells;
	d.clist_cap = (int) (cells / 8 + 8);
	d.rec = (double *) (base + NA_REC);
	d.tmp_rec = (double *) (base + NA_STAGE); /* float4 staging of the cell assignment */
	d.srec = (float4 *) (base + NA_SREC);
	d.id = (int *) (base + NA_ID);
	d.rep = (int *) (base + NA_REP);
	d.cellof = (int *) (base + NA_CELLOF);
	d.out_bonds = n_bonds_dev ? n_bonds_dev : (int *) (base + NA_BONDS);
	d.out_overlaps = n_overlaps_dev ? n_overlaps_dev : (int *) (base + NA_OVER);
	d.cell_count = (int *) (base + NA_CCOUNT);
	d.cell_start = (int *) (base + NA_CSTART);
	d.cell_cursor = (int *) (base + NA_CCURSOR);
	d.cell_rep = (int *) (base + NA_CREP);
	d.scan_aux = (int *) (base + NA_AUX);
	d.clist = (int *) (base + NA_CLIST);
	d.ccount = (int *) (base + NA_COLCOUNT);
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
			(c = cudaMemset(d.grid, 0, sizeof(ppi_grid))) != cudaSuccess || (c = cudaMemset(d.cell_rep, 0, sizeof(int) * (size_t) cells)) != cudaSuccess)
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
