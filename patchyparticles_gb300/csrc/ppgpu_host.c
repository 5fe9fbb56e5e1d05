/*
 * ppgpu_host.c -- C host side of the engine behind include/ppgpu.h: engine lifecycle, state upload /
 * download, the per-sweep launch sequence, energy checks, and the reference file formats (.rrr reader
 * and writer, seeded initial-configuration generator).
 *
 * Compiled with -ffp-contract=off: the .rrr reader must produce orientations bit-identical to the
 * reference's system_init (system.c:213-243), and the generator must reproduce generator.c.
 */
#define _GNU_SOURCE
#include "ppgpu.h"
#include "ppgpu_internal.h"

#include <cuda_runtime_api.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct pp_engine {
	int nrep;
	pp_params *prm;
	/* host-side staging of uploads until the device layout exists */
	int *N;
	double **h_r, **h_R;
	double (*h_box)[3];
	int *uploaded;
	int committed;
	/* device */
	ppi_dev d;
	ppi_rparams *h_rp;
	ppi_rstate *h_rs;
	int ntot_alloc;
	cudaStream_t stream;
	int threads;
	long long sweep_counter;
	long long round_counter;
	long long epoch;
	long long launches;
	int resort_every;     /* rounds between cell-grid re-sorts (new random shift, records rebuilt from FP64) */
	int rounds_per_sweep; /* checkerboard rounds per MC step */
	int reorder_every;    /* re-sorts between physical reorders of the FP64 state */
	double cell_scale;    /* cell edge / minimum edge (autotuner) */
	int any_npt;
	int any_lx;           /* some NVT replica has the box-shape move */
	int any_avb;          /* some replica makes AVB moves (Dynamics = 2) */
	int any_vmmc;         /* every replica makes VMMC moves (Dynamics = 1): no checkerboard rounds */
	int any_audit;
	int nl_mode;          /* per-epoch neighbour lists for plain moves (pp_gpu_set_neighbour_lists) */
	int nl_valid;         /* the current epoch's lists are built and only plain moves ran since */
	int nl_all;           /* every replica has lists (the volume pass then takes its pairs from them) */
	/* event timing */
	int timing;
	int n_ev;
	cudaEvent_t *ev;   /* groups of 2 events: start, stop */
	int *ev_kind;      /* 0 sort, 1 sweep, 2 volume */
	int ev_cap;
	pp_kernel_stats kstats;
	/* captured sweep graphs: one per re-sort period, with and without the physical reorder */
	int graphs_on;                /* pp_gpu_set_graphs (default 1) */
	int graphs_broken;            /* capture failed once: stream launches from then on */
	int graph_gen;                /* bumped whenever device pointers or the schedule change */
	cudaGraphExec_t gexec[2];
	cudaGraph_t gph[2];
	long long gnodes[2];
	int gkey[2][5];               /* resort_every, proposal, audit, npt, graph_gen of the capture */
	/* learned proposal */
	int learn_ready;              /* network buffers allocated (pp_gpu_learned_init) */
	int proposal;                 /* PP_PROPOSAL_PLAIN or PP_PROPOSAL_LEARNED */
	pp_learned_params lprm;
	ppi_learn h_learn;
	float *l_P, *l_m1, *l_m2, *l_grad; /* FP32 master weights, Adam moments, gradient (device) */
	unsigned char *l_img;         /* packed BF16 operands (device) */
	ppi_learn *l_learn;
	ppi_lrep *l_rep;              /* per replica mixture tables (device) */
	unsigned long long *l_stats;
	int *l_err;
	double *l_obj;
	int *l_tiles;
	int l_tiles_cap;
	long long n_samples;
	int adam_step;
	long long collect_snap;
	/* pinned staging */
	double *pin_rec;
	int *pin_id;
	int *pin_i1, *pin_i2;
	size_t pin_n;
	char err[512];
};

static int set_err(pp_engine *e, int code, const char *fmt, ...) {
	if(e) {
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(e->err, sizeof(e->err), fmt, ap);
		va_end(ap);
	}
	return code;
}

#define CU(call)                                                                                        \
	do {                                                                                                \
		cudaError_t _c = (call);                                                                        \
		if(_c != cudaSuccess) return set_err(e, PP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_c)); \
	} while(0)

#define CK(rc)                                                                                            \
	do {                                                                                                  \
		int _c = (rc);                                                                                    \
		if(_c != 0) return set_err(e, PP_ERR_CUDA, "kernel launch: %s", cudaGetErrorString((cudaError_t) _c)); \
	} while(0)

/* a host allocation that failed ends the call with PP_ERR_CAPACITY */
#define HOST_OK(ptr)                                                                   \
	do {                                                                               \
		if((ptr) == NULL) return set_err(e, PP_ERR_CAPACITY, "out of host memory: %s", #ptr); \
	} while(0)

/* ------------------------------------------------------------------------------------------------ */
/* small vector helpers with the reference's operation order (utils.c)                              */
/* ------------------------------------------------------------------------------------------------ */
#define H_SCALAR(x, y) ((x)[0] * (y)[0] + (x)[1] * (y)[1] + (x)[2] * (y)[2])

static void h_normalize(double *v) { /* utils.c:31-36 */
	double norm = sqrt(H_SCALAR(v, v));
	v[0] /= norm;
	v[1] /= norm;
	v[2] /= norm;
}

static void h_cross(const double *a, const double *b, double *r) { /* utils.c:25-29 */
	r[0] = a[1] * b[2] - a[2] * b[1];
	r[1] = a[2] * b[0] - a[0] * b[2];
	r[2] = a[0] * b[1] - a[1] * b[0];
}

static void h_gram_schmidt(double *v1, double *v2, double *v3) { /* utils.c:91-113 */
	double v1n = H_SCALAR(v1, v1);
	double b1 = H_SCALAR(v2, v1) / v1n;
	for(int k = 0; k < 3; k++) v2[k] -= b1 * v1[k];
	double v3v1 = H_SCALAR(v3, v1), v3v2 = H_SCALAR(v3, v2), v2n = H_SCALAR(v2, v2);
	b1 = v3v1 / v1n;
	double b2 = v3v2 / v2n;
	for(int k = 0; k < 3; k++) v3[k] -= b1 * v1[k] + b2 * v2[k];
	h_normalize(v1);
	h_normalize(v2);
	h_normalize(v3);
}

static void h_base_patches(double base[4][3]) { /* system.c:20-31 */
	double h = 0.5 / sqrt(3.);
	double v[4][3] = { { -h, -h, h }, { h, -h, -h }, { h, h, h }, { -h, h, -h } };
	for(int i = 0; i < 4; i++) {
		h_normalize(v[i]);
		memcpy(base[i], v[i], sizeof(v[i]));
	}
}

/* ------------------------------------------------------------------------------------------------ */
/* parameters                                                                                       */
/* ------------------------------------------------------------------------------------------------ */
void pp_default_params(pp_params *p) {
	memset(p, 0, sizeof(*p));
	p->ensemble = PP_NVT;
	p->temperature = 0.12;
	p->pressure = 0.;
	p->disp_max = 0.05;
	p->theta_max = 0.1;
	p->rescale_factor_max = 0.01;
	p->kf_delta = 0.12;
	p->kf_cosmax = 0.92;
	p->seed = 1;
	p->precision = PP_PREC_FP32_GUARD;
	p->guard_eps = 1e-5;
	p->resort_every = 0;
	p->audit = 0;
	p->dynamics = PP_RTMC;
	p->avb_p = 0.5; /* avb.c:30 */
	p->vmmc_max_cluster = 0;
	p->vmmc_max_move = 0.;
}

static int is_exchange(const pp_engine *e);

static int check_params(pp_engine *e, const pp_params *p) {
	if(p->ensemble != PP_NVT && p->ensemble != PP_NPT && p->ensemble != PP_GC && p->ensemble != PP_SUS)
		return set_err(e, PP_ERR_ARG, "Ensemble %d not supported (0 = NVT, 1 = GC, 3 = SUS, 5 = NPT)", p->ensemble);
	if(p->ensemble == PP_GC || p->ensemble == PP_SUS) {
		if(!(p->activity > 0.)) return set_err(e, PP_ERR_ARG, "Activity must be > 0");
		if(p->n_max < 1 || (p->ensemble == PP_SUS && (p->n_min < 0 || p->n_min > p->n_max)))
			return set_err(e, PP_ERR_ARG, "the particle-number window needs 0 <= Umbrella_sampling_min <= Umbrella_sampling_max and GC_N_max >= 1");
		if(p->lx_move) return set_err(e, PP_ERR_ARG, "Lx_move is not supported with insertions and removals");
	}
	if(!(p->temperature > 0.)) return set_err(e, PP_ERR_ARG, "Temperature must be > 0");
	if(!(p->disp_max >= 0.) || !(p->theta_max >= 0.)) return set_err(e, PP_ERR_ARG, "Disp_max and Theta_max must be >= 0");
	if(!(p->kf_delta > 0.) || !(p->kf_delta < 1.)) return set_err(e, PP_ERR_ARG, "KF_delta must lie in (0, 1)");
	if(!(p->kf_cosmax > -1.) || !(p->kf_cosmax < 1.)) return set_err(e, PP_ERR_ARG, "KF_cosmax must lie in (-1, 1)");
	if(p->precision != PP_PREC_FP32_GUARD && p->precision != PP_PREC_FP64) return set_err(e, PP_ERR_ARG, "unknown precision %d", p->precision);
	if(!(p->guard_eps <= 1e-2)) return set_err(e, PP_ERR_ARG, "guard_eps too large"); /* NaN too */
	if(p->resort_every < 0 || p->resort_every > 64) return set_err(e, PP_ERR_ARG, "resort_every (re-sort period in rounds) must be 0 or in [1, 64]");
	if(p->ensemble == PP_NPT && !(p->rescale_factor_max > 0. && p->rescale_factor_max < 1.)) return set_err(e, PP_ERR_ARG, "rescale_factor_max must lie in (0, 1)");
	if(p->lx_move < 0 || p->lx_move > 2) return set_err(e, PP_ERR_ARG, "Lx_move must be 0, 1 (reference acceptance) or 2 (Boltzmann acceptance)");
	if(p->dynamics != PP_RTMC && p->dynamics != PP_VMMC && p->dynamics != PP_AVBMC)
		return set_err(e, PP_ERR_ARG, "Dynamics %d not supported (0 = roto-translations, 1 = VMMC, 2 = AVB)", p->dynamics);
	if(p->dynamics == PP_VMMC) {
		if(p->ensemble != PP_NVT && p->ensemble != PP_NPT) return set_err(e, PP_ERR_ARG, "the VMMC move runs in the NVT and NPT ensembles");
		if(p->vmmc_max_cluster < 1) return set_err(e, PP_ERR_ARG, "vmmc_max_cluster must be >= 1");
	}
	if(p->dynamics == PP_AVBMC) {
		if(p->ensemble != PP_NVT && p->ensemble != PP_NPT) return set_err(e, PP_ERR_ARG, "the AVB move runs in the NVT and NPT ensembles");
		if(!(p->avb_p >= 0. && p->avb_p <= 1.)) return set_err(e, PP_ERR_ARG, "avb_p must lie in [0, 1]");
		if(sin(acos(p->kf_cosmax)) >= 1. / (2. * (1. + p->kf_delta))) /* avb.c:14-17 */
			return set_err(e, PP_ERR_ARG, "The AVB move cannot be used with patches that do not fulfill the single-bond-per-patch condition");
	}
	if(p->ensemble == PP_NVT && p->lx_move) {
		if(!(p->lx_change_max > 0.)) return set_err(e, PP_ERR_ARG, "Lx_change_max must be > 0");
		if(!(p->lyz_min > 0.) || !(p->lyz_max > p->lyz_min)) return set_err(e, PP_ERR_ARG, "Lyz_min and Lyz_max must satisfy 0 < Lyz_min < Lyz_max");
	}
	return PP_OK;
}

static int create_common(const pp_params *prms, int n, pp_engine **out) {
	if(out == NULL) return PP_ERR_ARG;
	*out = NULL;
	if(n < 1 || prms == NULL) return PP_ERR_ARG;
	pp_engine *e = calloc(1, sizeof(pp_engine));
	if(e == NULL) return PP_ERR_CAPACITY;
	for(int i = 0; i < n; i++) {
		int rc = check_params(e, prms + i);
		if(rc != PP_OK) {
			*out = e; /* let the caller read the message */
			e->nrep = 0;
			return rc;
		}
	}
	*out = e; /* from here on the caller can read the message, and destroy frees what was allocated */
	e->prm = calloc(n, sizeof(pp_params));
	e->N = calloc(n, sizeof(int));
	e->h_r = calloc(n, sizeof(double *));
	e->h_R = calloc(n, sizeof(double *));
	e->h_box = calloc(n, sizeof(double[3]));
	e->uploaded = calloc(n, sizeof(int));
	if(!e->prm || !e->N || !e->h_r || !e->h_R || !e->h_box || !e->uploaded) return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	e->nrep = n;
	memcpy(e->prm, prms, sizeof(pp_params) * n);
	e->threads = 128;
	e->resort_every = 4;
	e->rounds_per_sweep = 1;
	e->reorder_every = 16;
	e->cell_scale = 1.0;
	e->graphs_on = 1;
	e->nl_mode = 1;
	{ /* persistent round kernel: PPGPU_PERSIST=1 turns it on for every engine (pp_gpu_set_persistent per engine) */
		const char *v = getenv("PPGPU_PERSIST");
		e->d.persist = (v && atoi(v) == 1) ? 1 : 0;
	}
	for(int i = 0; i < n; i++) {
		if(e->prm[i].guard_eps <= 0.) e->prm[i].guard_eps = 1e-5;
		if(e->prm[i].ensemble == PP_NPT) e->any_npt = 1;
		if(e->prm[i].ensemble == PP_NVT && e->prm[i].lx_move) e->any_lx = 1;
		if(e->prm[i].audit) e->any_audit = 1;
		if(e->prm[i].dynamics == PP_AVBMC) e->any_avb = 1;
		if(e->prm[i].dynamics == PP_VMMC) e->any_vmmc = 1;
	}
	if(e->any_vmmc)
		for(int i = 0; i < n; i++)
			if(e->prm[i].dynamics != PP_VMMC) return set_err(e, PP_ERR_ARG, "VMMC replicas cannot share an engine with other dynamics");
	if(e->any_avb || e->any_vmmc) e->graphs_on = 0; /* the AVB / VMMC batches are launched from the host */
	if(e->prm[0].resort_every > 0) e->resort_every = e->prm[0].resort_every;
	for(int i = 0; i < n; i++)
		if((e->prm[i].ensemble == PP_GC || e->prm[i].ensemble == PP_SUS) && n > 1)
			return set_err(e, PP_ERR_ARG, "a GC or SUS system needs an engine of its own (pp_gpu_create)");
	if(is_exchange(e)) {
		/* the particle count changes between re-sorts: stream launches (a captured graph fixes it), and no
		 * physical reorder (it would interleave the live slots) */
		e->graphs_on = 0;
		e->reorder_every = 0;
	}
	cudaError_t c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
	*out = e;
	if(c != cudaSuccess) return set_err(e, PP_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(c));
	return PP_OK;
}

int pp_gpu_create(const pp_params *prm, pp_engine **out) { return create_common(prm, 1, out); }
int pp_gpu_create_batch(const pp_params *prms, int n, pp_engine **out) { return create_common(prms, n, out); }

const char *pp_gpu_last_error(const pp_engine *e) { return e ? e->err : "no engine"; }
int pp_gpu_num_replicas(const pp_engine *e) { return e ? e->nrep : 0; }
int pp_gpu_num_particles(const pp_engine *e, int r) { return (e && r >= 0 && r < e->nrep) ? e->N[r] : -1; }
long long pp_gpu_launch_count(const pp_engine *e) { return e ? e->launches : 0; }

static void drop_graphs(pp_engine *e);

static void free_device(pp_engine *e) {
	void **ptrs[] = { (void **) &e->d.rec, (void **) &e->d.spos, (void **) &e->d.sori, (void **) &e->d.id, (void **) &e->d.rep, (void **) &e->d.cellof,
		(void **) &e->d.cell_count, (void **) &e->d.cell_start, (void **) &e->d.cell_part, (void **) &e->d.cell_rep, (void **) &e->d.scan_aux,
		(void **) &e->d.clist, (void **) &e->d.ccount, (void **) &e->d.dflag, (void **) &e->d.eflag, (void **) &e->d.rp, (void **) &e->d.rs, (void **) &e->d.grid, (void **) &e->d.out_bonds,
		(void **) &e->d.out_overlaps, (void **) &e->d.out_partners, (void **) &e->d.tmp_rec, (void **) &e->d.tmp_id, (void **) &e->d.avb_head,
		(void **) &e->d.avb_next, (void **) &e->d.avb_cell, (void **) &e->d.vm_old, (void **) &e->d.vm_links, (void **) &e->d.vm_pre,
		(void **) &e->d.vm_fail, (void **) &e->d.vm_cnt, (void **) &e->d.vm_copies, (void **) &e->d.vm_in, (void **) &e->d.vm_clust };
	for(size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) {
		if(*ptrs[i]) cudaFree(*ptrs[i]);
		*ptrs[i] = NULL;
	}
	if(e->pin_rec) cudaFreeHost(e->pin_rec);
	if(e->pin_id) cudaFreeHost(e->pin_id);
	if(e->pin_i1) cudaFreeHost(e->pin_i1);
	if(e->pin_i2) cudaFreeHost(e->pin_i2);
	e->pin_rec = NULL;
	e->pin_id = e->pin_i1 = e->pin_i2 = NULL;
	e->pin_n = 0;
	if(e->d.ctr) cudaFree(e->d.ctr);
	e->d.ctr = NULL;
	if(e->d.gbar) cudaFree(e->d.gbar);
	e->d.gbar = NULL;
	if(e->d.sus_hist) cudaFree(e->d.sus_hist);
	e->d.sus_hist = NULL;
	if(e->d.nl) cudaFree(e->d.nl);
	if(e->d.nl_cnt) cudaFree(e->d.nl_cnt);
	if(e->d.vpairs) cudaFree(e->d.vpairs);
	if(e->d.vp_count) cudaFree(e->d.vp_count);
	if(e->d.srep) cudaFree(e->d.srep);
	if(e->d.vp_over) cudaFree(e->d.vp_over);
	if(e->d.vunsure) cudaFree(e->d.vunsure);
	if(e->d.vun_count) cudaFree(e->d.vun_count);
	e->d.nl = e->d.nl_cnt = e->d.vp_count = e->d.srep = e->d.vp_over = e->d.vun_count = NULL;
	e->d.vunsure = NULL;
	e->d.vun_cap = 0;
	e->d.vpairs = NULL;
	e->d.vp_cap = 0;
	e->d.nl_k = 0;
	e->nl_valid = 0;
	drop_graphs(e);
	/* layout-sized buffers of the learned proposal */
	if(e->d.simg) cudaFree(e->d.simg);
	if(e->d.feat) cudaFree(e->d.feat);
	e->d.simg = NULL;
	e->d.feat = NULL;
}

static void drop_graphs(pp_engine *e) {
	for(int v = 0; v < 2; v++) {
		if(e->gexec[v]) cudaGraphExecDestroy(e->gexec[v]);
		if(e->gph[v]) cudaGraphDestroy(e->gph[v]);
		e->gexec[v] = NULL;
		e->gph[v] = NULL;
	}
	e->graph_gen++;
}

static void free_learned(pp_engine *e) {
	void *ptrs[] = { e->l_P, e->l_m1, e->l_m2, e->l_grad, e->l_img, e->l_learn, e->l_rep, e->l_stats, e->l_err, e->l_obj, e->l_tiles, e->d.samples };
	for(size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++)
		if(ptrs[i]) cudaFree(ptrs[i]);
	e->l_P = e->l_m1 = e->l_m2 = e->l_grad = NULL;
	e->l_img = NULL;
	e->l_learn = NULL;
	e->l_rep = NULL;
	e->d.lrep = NULL;
	e->l_stats = NULL;
	e->l_err = NULL;
	e->l_obj = NULL;
	e->l_tiles = NULL;
	e->d.samples = NULL;
	e->d.sample_cap = 0;
	e->learn_ready = 0;
}

void pp_gpu_destroy(pp_engine *e) {
	if(e == NULL) return;
	if(e->stream) cudaStreamSynchronize(e->stream);
	free_device(e);
	free_learned(e);
	if(e->stream) cudaStreamDestroy(e->stream);
	for(int i = 0; i < e->nrep; i++) {
		free(e->h_r[i]);
		free(e->h_R[i]);
	}
	free(e->h_r);
	free(e->h_R);
	free(e->h_box);
	free(e->uploaded);
	free(e->N);
	free(e->prm);
	free(e->h_rp);
	free(e->h_rs);
	if(e->ev) {
		for(int i = 0; i < 2 * e->ev_cap; i++) cudaEventDestroy(e->ev[i]);
		free(e->ev);
		free(e->ev_kind);
	}
	free(e);
}

/* ------------------------------------------------------------------------------------------------ */
/* layout                                                                                           */
/* ------------------------------------------------------------------------------------------------ */
/* fills per-replica derived parameters; returns PP_OK or an error */
void ppi_model_params(int N, double kf_delta, double kf_cosmax, ppi_rparams *rp) {
	memset(rp, 0, sizeof(*rp));
	rp->N = N;
	rp->ensemble = PP_NVT;
	rp->T = 1.0;
	rp->cosmax = kf_cosmax;
	rp->sqr_rcut = (1. + kf_delta) * (1. + kf_delta); /* system.c:86 */
	rp->r_cut = 1. + kf_delta;                        /* system.c:249 */
	h_base_patches(rp->base);
	rp->w_min = rp->r_cut + 1e-5;
	rp->cosmax_f = (float) rp->cosmax;
	rp->sqr_rcut_f = (float) rp->sqr_rcut;
	rp->eps_f = 1e-5f;
	rp->base_f = (float) fabs(rp->base[0][0]);
	rp->seed = 1;
}

/* Bounds [smin, smax] of the factor by which one accepted box-shape move scales one side of the box of
 * replica r: an Lx move (MC.c:520-537) scales x by 1 +- Lx_change_max / (2 Lx) and y, z by sqrt(Lx / Lx'),
 * with Lx >= V / Lyz_max^2 (1, 1 without the move; NPT volume moves use exp(+-rescale_factor_max / 2)). */
static void lx_move_bounds(const pp_params *p, const double *box, double *smin, double *smax) {
	*smin = *smax = 1.;
	if(p->ensemble != PP_NVT || !p->lx_move) return;
	const double V = box[0] * box[1] * box[2], h = 0.5 * p->lx_change_max / (V / (p->lyz_max * p->lyz_max));
	*smin = fmin(1. - h, 1. / sqrt(1. + h));
	*smax = fmax(1. + h, 1. / sqrt(1. - h));
}

/* device slots of replica r: its particles, or for GC / SUS room for the largest allowed count */
static int slot_cap(const pp_engine *e, int r) {
	const pp_params *p = e->prm + r;
	if((p->ensemble == PP_GC || p->ensemble == PP_SUS) && p->n_max > e->N[r]) return p->n_max;
	return e->N[r];
}

static int is_exchange(const pp_engine *e) { return e->nrep == 1 && (e->prm[0].ensemble == PP_GC || e->prm[0].ensemble == PP_SUS); }

/* AVB (Dynamics = 2): AVBMC_init's volumes (avb.c:26-28) from the uploaded box, the attempts per MC step,
 * the linked-cell grid the batches may use, and a rotation base_orient taking base patch 0 to (0, 0, 1)
 * (system.c:33-54 builds one from random vectors; place_inside_vbonding follows it with a uniform turn
 * about base patch 0, so which one does not change the distribution of its orientations) */
static void avb_rparams(const pp_engine *e, int r, ppi_rparams *rp) {
	const pp_params *p = e->prm + r;
	const double *box = e->h_box[r];
	const double dl = p->kf_delta, cm = p->kf_cosmax;
	rp->avb_vin = 4 * 4 * (M_PI * (dl * dl * dl + 3. * (dl * dl) + 3. * dl) * ((1. - cm) * (1. - cm)) / 3.);
	rp->avb_vout = box[0] * box[1] * box[2] - rp->avb_vin;
	rp->avb_per_step = (int) floor((1. - p->avb_p) * e->N[r] + 0.5);
	const double grow = p->ensemble == PP_NPT ? 1.3 : 1.0;
	for(int a = 0; a < 3; a++) {
		int n = (int) floor(box[a] * grow / rp->r_cut);
		rp->avb_ncap[a] = n < 3 ? 3 : n;
	}
	const double *b0 = rp->base[0];
	double u[3] = { 1. - b0[0] * b0[0], -b0[0] * b0[1], -b0[0] * b0[2] }; /* e_x without its b0 part */
	const double nu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
	for(int k = 0; k < 3; k++) u[k] /= nu;
	const double v[3] = { b0[1] * u[2] - b0[2] * u[1], b0[2] * u[0] - b0[0] * u[2], b0[0] * u[1] - b0[1] * u[0] };
	for(int k = 0; k < 3; k++) {
		rp->base_orient[k] = u[k];
		rp->base_orient[3 + k] = v[k];
		rp->base_orient[6 + k] = b0[k];
	}
}

static int derive_rparams(pp_engine *e, int r, ppi_rparams *rp) {
	const pp_params *p = e->prm + r;
	memset(rp, 0, sizeof(*rp));
	rp->N = e->N[r];
	rp->ensemble = p->ensemble;
	rp->precision = p->precision;
	rp->audit = p->audit;
	rp->T = p->temperature;
	rp->P = p->pressure;
	rp->disp_max = p->disp_max;
	rp->theta_max = p->theta_max;
	rp->rescale_max = p->rescale_factor_max;
	rp->cosmax = p->kf_cosmax;
	rp->sqr_rcut = (1. + p->kf_delta) * (1. + p->kf_delta); /* system.c:86 */
	rp->r_cut = 1. + p->kf_delta;                           /* system.c:249 */
	h_base_patches(rp->base);
	/* cell edge: r_cut plus a margin for FP32 rounding of cell-local coordinates; NPT also leaves room for
	 * the accepted compressions between two re-sorts (each shrinks one side by at most exp(-max/2)) */
	double wm = rp->r_cut + 1e-5;
	if(p->ensemble == PP_NPT) wm /= exp(-0.5 * p->rescale_factor_max * (e->resort_every + 1));
	double lsmin, lsmax;
	lx_move_bounds(p, e->h_box[r], &lsmin, &lsmax);
	wm /= pow(lsmin, e->resort_every + 1); /* the Lx moves that can be accepted before the next re-sort */
	rp->w_min = wm * (e->cell_scale > 1.0 ? e->cell_scale : 1.0);
	rp->lx_move = (p->ensemble == PP_NVT) ? p->lx_move : 0;
	rp->lx_change_max = p->lx_change_max;
	rp->lyz_min = p->lyz_min;
	rp->lyz_max = p->lyz_max;
	rp->activity = p->activity;
	rp->n_min = p->ensemble == PP_SUS ? p->n_min : 0;
	rp->n_max = p->n_max;
	rp->dynamics = p->dynamics;
	rp->vmmc_max_cluster = p->vmmc_max_cluster;
	if(p->dynamics == PP_AVBMC || p->dynamics == PP_VMMC) avb_rparams(e, r, rp); /* the batches' linked cells */
	for(int k = 0; k < 32; k++) {
		double pk = exp(-(double) k / p->temperature);
		double t = ceil(pk * 9007199254740992.0);
		if(t > 9007199254740992.0) t = 9007199254740992.0;
		rp->acc_thr[k] = (uint64_t) t;
	}
	rp->cosmax_f = (float) rp->cosmax;
	rp->sqr_rcut_f = (float) rp->sqr_rcut;
	rp->eps_f = (float) p->guard_eps;
	rp->disp_max_f = (float) p->disp_max;
	rp->theta_max_f = (float) p->theta_max;
	rp->base_f = (float) fabs(rp->base[0][0]);
	rp->seed = p->seed;
	const double *box = e->h_box[r];
	double grow = (p->ensemble == PP_NPT) ? 1.15 : 1.0; /* a larger box is served by coarser cells */
	long long cap = 1;
	for(int a = 0; a < 3; a++) {
		int n = ((int) floor(box[a] / wm)) & ~1;
		if(n < 4) return set_err(e, PP_ERR_CAPACITY, "replica %d: box side %g is too small for the cell grid (needs >= 4 cells of edge %g)", r, box[a], wm);
		if(n > PPI_MAX_AXIS_CELLS) return set_err(e, PP_ERR_CAPACITY, "replica %d: box side %g needs more than %d cells", r, box[a], PPI_MAX_AXIS_CELLS);
		double side = box[a] * grow;
		if(rp->lx_move) /* the largest sides the box-shape move allows: Lx <= V / Lyz_min^2, Ly = Lz <= Lyz_max */
			side = a == 0 ? box[0] * box[1] * box[2] / (p->lyz_min * p->lyz_min) : p->lyz_max;
		int nc = ((int) floor(side / wm)) & ~1;
		if(nc > PPI_MAX_AXIS_CELLS) nc = PPI_MAX_AXIS_CELLS;
		cap *= nc;
	}
	if(cap > (1LL << 28)) return set_err(e, PP_ERR_CAPACITY, "replica %d: too many cells", r);
	rp->cell_cap = (int) cap;
	return PP_OK;
}

static int ensure_pinned(pp_engine *e, size_t n) {
	if(e->pin_n >= n && e->pin_rec) return PP_OK;
	if(e->pin_rec) cudaFreeHost(e->pin_rec);
	if(e->pin_id) cudaFreeHost(e->pin_id);
	if(e->pin_i1) cudaFreeHost(e->pin_i1);
	if(e->pin_i2) cudaFreeHost(e->pin_i2);
	e->pin_rec = NULL;
	e->pin_id = e->pin_i1 = e->pin_i2 = NULL;
	CU(cudaMallocHost((void **) &e->pin_rec, sizeof(double) * PPI_REC * (n ? n : 1)));
	CU(cudaMallocHost((void **) &e->pin_id, sizeof(int) * (n ? n : 1)));
	CU(cudaMallocHost((void **) &e->pin_i1, sizeof(int) * PPI_MAX_PARTNERS * (n ? n : 1)));
	CU(cudaMallocHost((void **) &e->pin_i2, sizeof(int) * (n ? n : 1)));
	e->pin_n = n;
	return PP_OK;
}

static int read_states(pp_engine *e) {
	CU(cudaMemcpyAsync(e->h_rs, e->d.rs, sizeof(ppi_rstate) * e->nrep, cudaMemcpyDeviceToHost, e->stream));
	int lerr = 0, berr = 0;
	if(e->learn_ready) CU(cudaMemcpyAsync(&lerr, e->l_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
	if(e->d.gbar) CU(cudaMemcpyAsync(&berr, e->d.gbar + 15, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	if(lerr) return set_err(e, PP_ERR_CUDA, "a tensor-core wait of the learned proposal timed out");
	if(berr == PPI_E_BARRIER) return set_err(e, PP_ERR_CUDA, "grid barrier wait timed out in the persistent round kernel (the state is incomplete)");
	for(int r = 0; r < e->nrep; r++)
		if(e->h_rs[r].error == PPI_E_GCFULL) /* MC.c:346-348 */
			return set_err(e, PP_ERR_CAPACITY, "The system contains the maximum number of particles set in the input file (%d), increase GC_N_max", e->prm[r].n_max);
	for(int r = 0; r < e->nrep; r++)
		if(e->h_rs[r].error == PPI_E_LISTS)
			return set_err(e, PP_ERR_CAPACITY, "replica %d: more guard-band pairs in one volume pass than its buffer holds", r);
		else if(e->h_rs[r].error == PPI_E_VMMC)
			return set_err(e, PP_ERR_STATE, "replica %d: VMMC: memory exhausted, or a cluster moved into an overlap", r);
		else if(e->h_rs[r].error == PPI_E_AVB)
			return set_err(e, PP_ERR_STATE, "replica %d: an AVB move's rejection sampling ran out of draws", r);
		else if(e->h_rs[r].error == PPI_E_EXACT)
			return set_err(e, PP_ERR_STATE, "replica %d: more pairs within 1e-12 of a bonding threshold than one warp keeps for the exact test", r);
		else if(e->h_rs[r].error)
			return set_err(e, PP_ERR_CAPACITY, "replica %d: the box no longer fits an even cell grid of edge >= r_cut (device error %d)", r, e->h_rs[r].error);
	return PP_OK;
}

static int write_states(pp_engine *e) {
	CU(cudaMemcpyAsync(e->d.rs, e->h_rs, sizeof(ppi_rstate) * e->nrep, cudaMemcpyHostToDevice, e->stream));
	return PP_OK;
}

static int do_resort(pp_engine *e) {
	long long nl = 0;
	if(e->reorder_every > 0 && e->epoch % e->reorder_every == 0) {
		/* physical reorder into the current cell order keeps the FP64 updates of a cell's particles local */
		CK(ppi_resort(&e->d, e->epoch, e->stream, &nl));
		CK(ppi_reorder(&e->d, e->stream, &nl));
	}
	CK(ppi_resort(&e->d, e->epoch, e->stream, &nl));
	if(e->proposal == PP_PROPOSAL_LEARNED && e->d.simg) CK(ppi_canon(&e->d, e->stream, &nl));
	e->nl_valid = 0;
	if(e->proposal == PP_PROPOSAL_PLAIN && e->d.nl_k > 0) {
		CK(ppi_nlist(&e->d, e->stream, &nl));
		e->nl_valid = 1;
	}
	e->launches += nl;
	e->epoch++;
	return PP_OK;
}

/* energy of every replica from scratch into rs.vol_bonds / vol_overlap (per-slot counts in out_*) */
static int run_energy(pp_engine *e, int mode) {
	long long nl = 0;
	CK(ppi_energy(&e->d, mode, e->stream, &nl));
	e->launches += nl;
	return read_states(e);
}

/* Squared radius of replica r's neighbour lists. Between two re-sorts (at most resort_every rounds) each
 * particle moves at most once per round by |d| <= sqrt(3)/2 Disp_max, so a pair's separation changes by at
 * most sqrt(3) Disp_max per round; NPT adds the accepted rescalings (each scales one axis by a factor in
 * [exp(-max/2), exp(max/2)], at most one per round, and one more for the candidate box). A pair farther
 * apart than the radius at the re-sort therefore stays beyond r_cut + 1e-3 and outside the FP32 guard band
 * on r^2 for the whole epoch. FP64-precision replicas get no lists (every pair takes the exact path). */
static float nl_radius2(const pp_engine *e, int r) {
	const pp_params *p = e->prm + r;
	if(p->precision == PP_PREC_FP64) return 0.f;
	const double E = (double) e->resort_every, rc = 1. + p->kf_delta;
	const double base = sqrt((rc + 1e-3) * (rc + 1e-3) + p->guard_eps);
	const double motion = sqrt(3.) * E * p->disp_max;
	double R = base + motion;
	if(p->ensemble == PP_NPT) {
		const double smin = exp(-0.5 * p->rescale_factor_max * (E + 1.)), smax = exp(0.5 * p->rescale_factor_max * E);
		R = (base + smax * motion) / smin;
	}
	else if(p->lx_move) { /* the same for the Lx moves of the epoch (MC.c:520-545) */
		double s1, s2;
		lx_move_bounds(p, e->h_box[r], &s1, &s2);
		R = (base + pow(s2, E) * motion) / pow(s1, E + 1.);
	}
	R += 1e-3;
	return (float) (R * R * (1. + 1e-6));
}

/* Radii of every replica and the per-particle list capacity (a generous bound on the listed count at the
 * replica's density, 1.5x the density for NPT); (re)allocates the lists when the capacity grows. A list
 * that overflows anyway sends its particle's attempts to the exact 27-cell path. */
static int setup_nlists(pp_engine *e) {
	int K = 0;
	e->nl_all = 1;
	for(int r = 0; r < e->nrep; r++) {
		e->h_rp[r].nl_r2f = e->nl_mode ? nl_radius2(e, r) : 0.f;
		if(!(e->h_rp[r].nl_r2f > 0.f)) {
			e->nl_all = 0;
			continue;
		}
		const double R = sqrt((double) e->h_rp[r].nl_r2f), *b = e->h_box[r];
		double rho = slot_cap(e, r) / (b[0] * b[1] * b[2]);
		if(e->prm[r].ensemble == PP_NPT) rho *= 1.5;
		const double mean = 4.18879020478639 * R * R * R * rho;
		int k = (int) ceil(mean + 6. * sqrt(mean) + 6.);
		if(k > K) K = k;
	}
	if(K > 0) K = K < 8 ? 8 : (K > 128 ? 128 : (K + 3) & ~3);
	{ /* a capacity override for tests of the overflow path (PPGPU_NL_CAP, rounded up to a multiple of 4) */
		const char *v = getenv("PPGPU_NL_CAP");
		if(K > 0 && v && atoi(v) > 0 && atoi(v) <= 128) K = (atoi(v) + 3) & ~3;
	}
	if(!e->nl_mode || e->d.ntot >= (1 << 27)) K = 0; /* a list entry holds sorted positions below 2^27 */
	/* (re)allocate when the capacity grows; K == 0 frees the lists */
	if(K == 0 && e->d.nl_k == 0 && e->d.nl == NULL) return PP_OK;
	if(K > 0 && K <= e->d.nl_k && e->d.nl != NULL) return PP_OK;
	drop_graphs(e);
	e->graph_gen++;
	if(e->d.nl) cudaFree(e->d.nl);
	if(e->d.nl_cnt) cudaFree(e->d.nl_cnt);
	if(e->d.vpairs) cudaFree(e->d.vpairs);
	if(e->d.vp_count) cudaFree(e->d.vp_count);
	if(e->d.srep) cudaFree(e->d.srep);
	if(e->d.vp_over) cudaFree(e->d.vp_over);
	if(e->d.vunsure) cudaFree(e->d.vunsure);
	if(e->d.vun_count) cudaFree(e->d.vun_count);
	e->d.nl = e->d.nl_cnt = e->d.vp_count = e->d.srep = e->d.vp_over = e->d.vun_count = NULL;
	e->d.vunsure = NULL;
	e->d.vun_cap = 0;
	e->d.vpairs = NULL;
	e->d.vp_cap = 0;
	e->d.nl_k = 0;
	e->nl_valid = 0;
	if(K == 0) return PP_OK;
	const size_t n1 = e->ntot_alloc > 0 ? (size_t) e->ntot_alloc : 1;
	CU(cudaMalloc((void **) &e->d.nl, sizeof(int) * (size_t) K * n1));
	CU(cudaMalloc((void **) &e->d.nl_cnt, sizeof(int) * n1));
	/* the volume pass's flat pair list: at most K pairs above each particle (an overflowing particle goes to
	 * vp_over), so the capacity cannot run out */
	if((size_t) K * n1 < (size_t) 1 << 31) {
		CU(cudaMalloc((void **) &e->d.vpairs, sizeof(int2) * (size_t) K * n1));
		CU(cudaMalloc((void **) &e->d.vp_count, 2 * sizeof(int)));
		CU(cudaMalloc((void **) &e->d.srep, sizeof(int) * n1));
		CU(cudaMalloc((void **) &e->d.vp_over, sizeof(int) * n1));
		CU(cudaMemsetAsync(e->d.vp_count, 0, 2 * sizeof(int), e->stream));
		e->d.vp_cap = (int) ((size_t) K * n1);
		/* guard-band pairs of one volume pass (a fraction ~eps of the close pairs; FP64 replicas have no lists) */
		e->d.vun_cap = (int) (n1 + 65536);
		CU(cudaMalloc((void **) &e->d.vunsure, sizeof(int2) * (size_t) e->d.vun_cap));
		CU(cudaMalloc((void **) &e->d.vun_count, sizeof(int)));
	}
	e->d.nl_k = K;
	return PP_OK;
}

static int commit(pp_engine *e) {
	int ntot = 0, nalloc = 0;
	for(int r = 0; r < e->nrep; r++) {
		ntot += e->N[r];
		nalloc += slot_cap(e, r);
	}
	e->ntot_alloc = nalloc;
	free_device(e);
	free(e->h_rp);
	free(e->h_rs);
	e->h_rp = calloc(e->nrep, sizeof(ppi_rparams));
	e->h_rs = calloc(e->nrep, sizeof(ppi_rstate));
	HOST_OK(e->h_rp);
	HOST_OK(e->h_rs);
	long long cells = 0, avb_cells = 0;
	int p0 = 0;
	for(int r = 0; r < e->nrep; r++) {
		ppi_rparams *rp = e->h_rp + r;
		int rc = derive_rparams(e, r, rp);
		if(rc != PP_OK) return rc;
		rp->p0 = p0;
		p0 += slot_cap(e, r);
		rp->cell_base = (int) cells;
		cells += rp->cell_cap;
		if(rp->dynamics == PP_AVBMC || rp->dynamics == PP_VMMC) {
			rp->avb_head0 = (int) avb_cells;
			avb_cells += (long long) rp->avb_ncap[0] * rp->avb_ncap[1] * rp->avb_ncap[2];
		}
	}
	if(avb_cells > (1LL << 30)) return set_err(e, PP_ERR_CAPACITY, "too many AVB cells in total");
	if(cells > (1LL << 30)) return set_err(e, PP_ERR_CAPACITY, "too many cells in total");
	ppi_dev *d = &e->d;
	d->nrep = e->nrep;
	d->ntot = ntot;
	d->total_cells = (int) cells;
	d->clist_cap = (int) (cells / 8 + e->nrep + 8);
	size_t n1 = nalloc > 0 ? (size_t) nalloc : 1;
	CU(cudaMalloc((void **) &d->rec, sizeof(double) * PPI_REC * n1));
	CU(cudaMalloc((void **) &d->spos, sizeof(float) * 4 * n1));
	CU(cudaMalloc((void **) &d->sori, sizeof(float) * 12 * n1));
	CU(cudaMalloc((void **) &d->id, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->rep, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->cellof, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->out_bonds, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->out_overlaps, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->out_partners, sizeof(int) * PPI_MAX_PARTNERS * n1));
	CU(cudaMalloc((void **) &d->tmp_rec, sizeof(double) * PPI_REC * n1));
	CU(cudaMalloc((void **) &d->tmp_id, sizeof(int) * n1));
	CU(cudaMalloc((void **) &d->cell_count, sizeof(int) * cells));
	CU(cudaMalloc((void **) &d->cell_start, sizeof(int) * (cells + 1)));
	CU(cudaMalloc((void **) &d->cell_part, sizeof(int) * cells));
	CU(cudaMalloc((void **) &d->cell_rep, sizeof(int) * cells));
	CU(cudaMalloc((void **) &d->scan_aux, sizeof(int) * ((cells + 1023) / 1024 + 1)));
	CU(cudaMalloc((void **) &d->clist, sizeof(int4) * 8 * (size_t) d->clist_cap));
	CU(cudaMalloc((void **) &d->ccount, sizeof(int) * 16)); /* 8 colour counts, the scan ticket */
	CU(cudaMalloc((void **) &d->dflag, 8 * (size_t) d->clist_cap));
	CU(cudaMemsetAsync(d->dflag, 0, 8 * (size_t) d->clist_cap, e->stream));
	CU(cudaMalloc((void **) &d->eflag, n1));
	CU(cudaMemsetAsync(d->eflag, 0, n1, e->stream));
	if(avb_cells > 0) {
		CU(cudaMalloc((void **) &d->avb_head, sizeof(int) * (size_t) avb_cells));
		CU(cudaMalloc((void **) &d->avb_next, sizeof(int) * n1));
		CU(cudaMalloc((void **) &d->avb_cell, sizeof(int) * n1));
	}
	if(e->any_vmmc) { /* VMMC_init's arrays (vmmc.c:28-42), 16 links per particle */
		CU(cudaMalloc((void **) &d->vm_old, sizeof(double) * 12 * n1));
		CU(cudaMalloc((void **) &d->vm_links, sizeof(int) * 2 * 16 * n1));
		CU(cudaMalloc((void **) &d->vm_pre, sizeof(int) * 16 * n1));
		CU(cudaMalloc((void **) &d->vm_fail, sizeof(int) * 16 * n1));
		CU(cudaMalloc((void **) &d->vm_cnt, sizeof(int) * n1));
		CU(cudaMalloc((void **) &d->vm_copies, sizeof(int) * n1));
		CU(cudaMalloc((void **) &d->vm_in, sizeof(int) * n1));
		CU(cudaMalloc((void **) &d->vm_clust, sizeof(int) * n1));
	}
	d->audit_any = e->any_audit;
	{ /* lanes per attempt: a tuning override for measurements (4 by default) */
		const char *v = getenv("PPGPU_LANES");
		d->lanes = (v && atoi(v) == 8) ? 8 : 4;
	}
	CU(cudaMalloc((void **) &d->rp, sizeof(ppi_rparams) * e->nrep));
	CU(cudaMalloc((void **) &d->rs, sizeof(ppi_rstate) * e->nrep));
	CU(cudaMalloc((void **) &d->grid, sizeof(ppi_grid) * e->nrep));
	CU(cudaMalloc((void **) &d->ctr, sizeof(ppi_ctr)));
	CU(cudaMalloc((void **) &d->gbar, 16 * sizeof(int)));
	CU(cudaMemsetAsync(d->gbar, 0, 16 * sizeof(int), e->stream));
	CU(cudaMemsetAsync(d->out_bonds, 0, sizeof(int) * n1, e->stream));
	CU(cudaMemsetAsync(d->out_overlaps, 0, sizeof(int) * n1, e->stream));
	CU(cudaMemsetAsync(d->grid, 0, sizeof(ppi_grid) * e->nrep, e->stream));
	int rc = ensure_pinned(e, n1);
	if(rc != PP_OK) return rc;
	rc = setup_nlists(e);
	if(rc != PP_OK) return rc;
	int *crep = malloc(sizeof(int) * (cells > 0 ? cells : 1));
	int *rep = malloc(sizeof(int) * n1);
	if(crep == NULL || rep == NULL) {
		free(crep);
		free(rep);
		return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	}
	for(int r = 0; r < e->nrep; r++) {
		ppi_rparams *rp = e->h_rp + r;
		for(int c = 0; c < rp->cell_cap; c++) crep[rp->cell_base + c] = r;
		for(int i = 0; i < slot_cap(e, r); i++) rep[rp->p0 + i] = r;
	}
	cudaError_t c1 = cudaMemcpy(d->cell_rep, crep, sizeof(int) * cells, cudaMemcpyHostToDevice);
	cudaError_t c2 = cudaMemcpy(d->rep, rep, sizeof(int) * n1, cudaMemcpyHostToDevice);
	free(crep);
	free(rep);
	if(c1 != cudaSuccess || c2 != cudaSuccess) return set_err(e, PP_ERR_CUDA, "layout upload failed");
	if(is_exchange(e)) {
		const pp_params *p = e->prm;
		const int nb = (p->ensemble == PP_SUS ? p->n_max - p->n_min : p->n_max) + 1;
		CU(cudaMalloc((void **) &d->sus_hist, sizeof(unsigned long long) * (size_t) nb));
		CU(cudaMemsetAsync(d->sus_hist, 0, sizeof(unsigned long long) * (size_t) nb, e->stream));
	}
	CU(cudaMemcpy(d->rp, e->h_rp, sizeof(ppi_rparams) * e->nrep, cudaMemcpyHostToDevice));
	e->committed = 1;
	return PP_OK;
}

/* all-ones exponent: an infinity or a NaN */
static inline uint64_t nonfinite_bits(double v) {
	uint64_t u;
	memcpy(&u, &v, sizeof(u));
	return ((u >> 52) & 0x7ff) == 0x7ff;
}

/* copies replica r's host arrays into its device slots. A non-finite coordinate or orientation entry
 * (checked in the same pass) refuses the upload: the replica is then without a configuration until the
 * next upload. */
static int push_replica(pp_engine *e, int r, const double *rr, const double *RR) {
	ppi_rparams *rp = e->h_rp + r;
	int N = rp->N;
	uint64_t bad = 0;
	for(int i = 0; i < N; i++) {
		double *dst = e->pin_rec + (size_t) i * PPI_REC;
		dst[0] = rr[3 * i];
		dst[1] = rr[3 * i + 1];
		dst[2] = rr[3 * i + 2];
		dst[PPI_Q] = 1.0; /* accumulated rotation: identity, so R = R0 is the uploaded matrix bit for bit */
		dst[PPI_Q + 1] = 0.0;
		dst[PPI_Q + 2] = 0.0;
		dst[PPI_Q + 3] = 0.0;
		memcpy(dst + PPI_R0, RR + 9 * (size_t) i, 9 * sizeof(double));
		for(int k = 0; k < 3; k++) bad |= nonfinite_bits(dst[k]);
		for(int k = 0; k < 9; k++) bad |= nonfinite_bits(dst[PPI_R0 + k]);
		e->pin_id[i] = i;
	}
	if(bad) {
		e->committed = 0;
		e->uploaded[r] = 0;
		return set_err(e, PP_ERR_ARG, "replica %d: a position or orientation entry is not finite", r);
	}
	CU(cudaMemcpyAsync(e->d.rec + (size_t) rp->p0 * PPI_REC, e->pin_rec, sizeof(double) * PPI_REC * N, cudaMemcpyHostToDevice, e->stream));
	CU(cudaMemcpyAsync(e->d.id + rp->p0, e->pin_id, sizeof(int) * N, cudaMemcpyHostToDevice, e->stream));
	/* the pinned buffer is reused by the next replica: wait for this copy */
	CU(cudaStreamSynchronize(e->stream));
	return PP_OK;
}

/* state uploaded: cell sort (with a physical reorder), initial energy and overlap check (main.c:55-64) */
static int finish_upload(pp_engine *e, int only) {
	int rc;
	long long nl = 0;
	CK(ppi_resort(&e->d, e->epoch, e->stream, &nl));
	CK(ppi_reorder(&e->d, e->stream, &nl));
	e->launches += nl;
	rc = do_resort(e);
	if(rc != PP_OK) return rc;
	rc = run_energy(e, PPI_EN_BONDS);
	if(rc != PP_OK) return rc;
	int bad = -1;
	for(int r = 0; r < e->nrep; r++) {
		if(only >= 0 && r != only) continue;
		ppi_rstate *s = e->h_rs + r;
		if(s->vol_overlap && bad < 0) bad = r;
		s->bonds = s->vol_bonds / 2;
		s->pairs = s->fallbacks = 0;
	}
	rc = write_states(e);
	if(rc != PP_OK) return rc;
	CU(cudaStreamSynchronize(e->stream));
	if(bad >= 0) return set_err(e, PP_ERR_OVERLAP, "Initial configuration contains an overlap, aborting (replica %d)", bad);
	return PP_OK;
}

int pp_gpu_upload_replica(pp_engine *e, int r, int N, const double *rr, const double *RR, const double box[3]) {
	if(e == NULL || r < 0 || r >= e->nrep || N < 0 || (N > 0 && (rr == NULL || RR == NULL)) || box == NULL) return set_err(e, PP_ERR_ARG, "invalid upload arguments");
	for(int a = 0; a < 3; a++)
		if(!(box[a] > 0.) || nonfinite_bits(box[a])) return set_err(e, PP_ERR_ARG, "box sides must be positive and finite");
	const pp_params *p = e->prm + r;
	if(p->ensemble == PP_SUS) { /* system.c:100-101 */
		if(N < p->n_min) return set_err(e, PP_ERR_ARG, "Number of particles %d is smaller than Umbrella_sampling_min (%d)", N, p->n_min);
		if(N > p->n_max) return set_err(e, PP_ERR_ARG, "Number of particles %d is larger than Umbrella_sampling_max (%d)", N, p->n_max);
	}
	if(p->ensemble == PP_GC && N > p->n_max) return set_err(e, PP_ERR_ARG, "Number of particles %d is larger than GC_N_max (%d)", N, p->n_max);
	if(p->ensemble == PP_NVT && p->lx_move) { /* system.c:172-188 */
		if(box[1] != box[2]) return set_err(e, PP_ERR_ARG, "Lx_move = 1 requires Ly = Lz");
		if(p->lyz_min >= box[1]) return set_err(e, PP_ERR_ARG, "Lyz_min should be smaller than box size");
		if(p->lyz_max <= box[1]) return set_err(e, PP_ERR_ARG, "Lyz_max should be larger than box size");
		if(0.5 * p->lx_change_max >= 0.5 * box[0] * box[1] * box[2] / (p->lyz_max * p->lyz_max))
			return set_err(e, PP_ERR_ARG, "Lx_change_max is too large: one move could halve the smallest Lx that Lyz_max allows");
	}
	/* fast path: same layout already on the device -> copy straight into the replica's slots */
	if(e->committed && e->N[r] == N) {
		double grow = (e->prm[r].ensemble == PP_NPT) ? 1.15 : 1.0;
		long long cap = 1;
		for(int a = 0; a < 3; a++) {
			int nc = ((int) floor(box[a] * grow / e->h_rp[r].w_min)) & ~1;
			cap *= nc < 4 ? 4 : nc;
		}
		if(cap <= e->h_rp[r].cell_cap) {
			int rc = read_states(e);
			if(rc != PP_OK) return rc;
			memcpy(e->h_box[r], box, sizeof(double) * 3);
			if(e->prm[r].dynamics == PP_AVBMC || e->prm[r].dynamics == PP_VMMC) { /* AVBMC_init's V_out follows the uploaded box; the cell grid keeps its reservation */
				ppi_rparams *rp = e->h_rp + r;
				int ncap[3] = { rp->avb_ncap[0], rp->avb_ncap[1], rp->avb_ncap[2] };
				avb_rparams(e, r, rp);
				for(int a = 0; a < 3; a++) rp->avb_ncap[a] = ncap[a];
				CU(cudaMemcpy(e->d.rp + r, rp, sizeof(ppi_rparams), cudaMemcpyHostToDevice));
			}
			ppi_rstate *s = e->h_rs + r;
			memset(s, 0, sizeof(*s));
			memcpy(s->box, box, sizeof(s->box));
			s->V = box[0] * box[1] * box[2];
			s->n_live = N;
			rc = write_states(e);
			if(rc != PP_OK) return rc;
			rc = push_replica(e, r, rr, RR);
			if(rc != PP_OK) return rc;
			return finish_upload(e, r);
		}
	}
	free(e->h_r[r]);
	free(e->h_R[r]);
	e->h_r[r] = malloc(sizeof(double) * 3 * (N > 0 ? N : 1));
	e->h_R[r] = malloc(sizeof(double) * 9 * (N > 0 ? N : 1));
	HOST_OK(e->h_r[r]);
	HOST_OK(e->h_R[r]);
	if(N > 0) {
		memcpy(e->h_r[r], rr, sizeof(double) * 3 * N);
		memcpy(e->h_R[r], RR, sizeof(double) * 9 * N);
	}
	memcpy(e->h_box[r], box, sizeof(double) * 3);
	e->N[r] = N;
	e->uploaded[r] = 1;
	e->committed = 0;
	for(int q = 0; q < e->nrep; q++)
		if(!e->uploaded[q]) return PP_OK; /* wait for the rest of the batch */
	int rc = commit(e);
	if(rc != PP_OK) return rc;
	for(int q = 0; q < e->nrep; q++) {
		ppi_rstate *s = e->h_rs + q;
		memset(s, 0, sizeof(*s));
		memcpy(s->box, e->h_box[q], sizeof(s->box));
		s->V = s->box[0] * s->box[1] * s->box[2];
		s->n_live = e->N[q];
	}
	rc = write_states(e);
	if(rc != PP_OK) return rc;
	for(int q = 0; q < e->nrep; q++) {
		rc = push_replica(e, q, e->h_r[q], e->h_R[q]);
		if(rc != PP_OK) return rc;
	}
	return finish_upload(e, -1);
}

int pp_gpu_upload(pp_engine *e, int N, const double *r, const double *R, const double box[3]) { return pp_gpu_upload_replica(e, 0, N, r, R, box); }

static int ready(pp_engine *e) {
	if(e == NULL) return PP_ERR_ARG;
	if(!e->committed) return set_err(e, PP_ERR_STATE, "no configuration uploaded for every replica");
	return PP_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* event timing                                                                                     */
/* ------------------------------------------------------------------------------------------------ */
static int collect_events(pp_engine *e) {
	if(e->n_ev == 0) return PP_OK;
	CU(cudaStreamSynchronize(e->stream));
	for(int i = 0; i < e->n_ev; i++) {
		float ms = 0.f;
		CU(cudaEventElapsedTime(&ms, e->ev[2 * i], e->ev[2 * i + 1]));
		if(e->ev_kind[i] == 0) {
			e->kstats.sort_ms += ms;
			e->kstats.sort_launches++;
		}
		else if(e->ev_kind[i] == 1) {
			e->kstats.sweep_ms += ms;
			e->kstats.sweep_launches++;
		}
		else {
			e->kstats.volume_ms += ms;
			e->kstats.volume_launches++;
		}
	}
	e->n_ev = 0;
	return PP_OK;
}

static int ev_begin(pp_engine *e, int kind, int *slot) {
	*slot = -1;
	if(!e->timing) return PP_OK;
	if(e->n_ev == e->ev_cap) {
		int rc = collect_events(e);
		if(rc != PP_OK) return rc;
	}
	int i = e->n_ev++;
	e->ev_kind[i] = kind;
	CU(cudaEventRecord(e->ev[2 * i], e->stream));
	*slot = i;
	return PP_OK;
}

static int ev_end(pp_engine *e, int slot) {
	if(slot < 0) return PP_OK;
	CU(cudaEventRecord(e->ev[2 * slot + 1], e->stream));
	return PP_OK;
}

int pp_gpu_set_timing(pp_engine *e, int enable) {
	if(e == NULL) return PP_ERR_ARG;
	if(enable && e->ev == NULL) {
		e->ev_cap = 3072;
		e->ev = calloc(2 * e->ev_cap, sizeof(cudaEvent_t));
		e->ev_kind = calloc(e->ev_cap, sizeof(int));
		if(e->ev == NULL || e->ev_kind == NULL) {
			free(e->ev);
			free(e->ev_kind);
			e->ev = NULL;
			e->ev_kind = NULL;
			e->ev_cap = 0;
			return set_err(e, PP_ERR_CAPACITY, "out of host memory");
		}
		for(int i = 0; i < 2 * e->ev_cap; i++) CU(cudaEventCreate(&e->ev[i]));
	}
	if(!enable) {
		int rc = collect_events(e);
		if(rc != PP_OK) return rc;
	}
	e->timing = enable ? 1 : 0;
	return PP_OK;
}

int pp_gpu_kernel_stats(pp_engine *e, pp_kernel_stats *out, int reset) {
	if(e == NULL) return PP_ERR_ARG;
	int rc = collect_events(e);
	if(rc != PP_OK) return rc;
	if(out) *out = e->kstats;
	if(reset) memset(&e->kstats, 0, sizeof(e->kstats));
	return PP_OK;
}

int pp_gpu_select_device(int device) {
	cudaError_t c = cudaSetDevice(device);
	return c == cudaSuccess ? PP_OK : PP_ERR_CUDA;
}

/* ------------------------------------------------------------------------------------------------ */
/* sweeps                                                                                           */
/* ------------------------------------------------------------------------------------------------ */
/* order of the 8 checkerboard colours in a round: a Fisher-Yates shuffle driven by splitmix64 of the round
 * index. It depends on no replica's seed, so a replica's trajectory does not depend on its batch. */
static void colour_order(long long round, int col[8]) {
	uint64_t z = (uint64_t) round * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
	for(int i = 0; i < 8; i++) col[i] = i;
	for(int i = 7; i > 0; i--) {
		z += 0x9E3779B97F4A7C15ULL;
		uint64_t x = z;
		x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
		x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
		x ^= x >> 31;
		int j = (int) (x % (uint64_t) (i + 1));
		int t = col[i];
		col[i] = col[j];
		col[j] = t;
	}
}

/* One MC step: `rounds_per_sweep` checkerboard rounds (one attempt per non-empty cell per round, the
 * grid re-sorted from the FP64 state every resort_every rounds), then one NPT volume attempt. */
#define GRAPH_UNAVAILABLE 1 /* internal: capture not possible, use stream launches */

/* Captures one re-sort period (the re-sort, with the physical reorder if v, then resort_every rounds, each
 * followed by the NPT volume attempt) as a CUDA graph whose launches read the round / epoch / sweep
 * indices from the device counters. The launches are the stream path's, argument for argument. */
static int capture_period(pp_engine *e, int v) {
	const int R = e->resort_every, learned = e->proposal == PP_PROPOSAL_LEARNED;
	static const int slots[8] = { 0, 1, 2, 3, 4, 5, 6, 7 };
	if(ppi_prepare(&e->d) != 0) {
		cudaGetLastError();
		return GRAPH_UNAVAILABLE;
	}
	long long nl = 0;
	cudaGraph_t g = NULL;
	if(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		cudaGetLastError();
		return GRAPH_UNAVAILABLE;
	}
	int rc = 0;
	if(v) {
		rc |= ppi_resort(&e->d, -1, e->stream, &nl);
		rc |= ppi_reorder(&e->d, e->stream, &nl);
	}
	rc |= ppi_resort(&e->d, -1, e->stream, &nl);
	if(learned) rc |= ppi_canon(&e->d, e->stream, &nl);
	const int lists = !learned && e->d.nl_k > 0;
	if(lists) rc |= ppi_nlist(&e->d, e->stream, &nl);
	for(int r = 0; r < R; r++) {
		if(learned) rc |= ppi_round_learned(&e->d, -1 - r, slots, e->any_audit, e->stream, &nl);
		else rc |= ppi_round(&e->d, -1 - r, slots, e->any_audit, lists, e->stream, &nl);
		if(e->any_npt || e->any_lx) {
			rc |= ppi_volume(&e->d, -1 - r, lists && e->nl_all, e->stream, &nl);
			if(learned) rc |= ppi_canon(&e->d, e->stream, &nl);
		}
	}
	const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
	cudaGraphExec_t x = NULL;
	if(rc != 0 || ce != cudaSuccess || g == NULL || cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
		if(g) cudaGraphDestroy(g);
		cudaGetLastError();
		return GRAPH_UNAVAILABLE;
	}
	e->gexec[v] = x;
	e->gph[v] = g;
	e->gnodes[v] = nl;
	e->gkey[v][0] = R;
	e->gkey[v][1] = e->proposal;
	e->gkey[v][2] = e->any_audit;
	e->gkey[v][3] = e->any_npt;
	e->gkey[v][4] = e->graph_gen;
	return PP_OK;
}

/* one re-sort period (resort_every sweeps) by replaying its graph */
static int replay_period(pp_engine *e) {
	const int v = (e->reorder_every > 0 && e->epoch % e->reorder_every == 0) ? 1 : 0;
	if(e->gexec[v] && (e->gkey[v][0] != e->resort_every || e->gkey[v][1] != e->proposal || e->gkey[v][2] != e->any_audit || e->gkey[v][3] != e->any_npt ||
							  e->gkey[v][4] != e->graph_gen)) {
		cudaGraphExecDestroy(e->gexec[v]);
		cudaGraphDestroy(e->gph[v]);
		e->gexec[v] = NULL;
		e->gph[v] = NULL;
	}
	if(!e->gexec[v]) {
		const int rc = capture_period(e, v);
		if(rc != PP_OK) return rc;
	}
	long long nl = 0;
	CK(ppi_set_counters(&e->d, e->round_counter, e->epoch, e->sweep_counter, e->stream, &nl));
	CU(cudaGraphLaunch(e->gexec[v], e->stream));
	e->nl_valid = e->proposal == PP_PROPOSAL_PLAIN && e->d.nl_k > 0;
	e->launches += nl + e->gnodes[v];
	e->round_counter += e->resort_every;
	e->sweep_counter += e->resort_every;
	e->epoch++;
	return PP_OK;
}

int pp_gpu_set_neighbour_lists(pp_engine *e, int enable) {
	if(e == NULL) return PP_ERR_ARG;
	enable = enable ? 1 : 0;
	if(enable == e->nl_mode) return PP_OK;
	e->nl_mode = enable;
	if(!e->committed) return PP_OK;
	int rc = setup_nlists(e);
	if(rc != PP_OK) return rc;
	drop_graphs(e);
	e->graph_gen++;
	e->nl_valid = 0; /* lists are (re)built at the next re-sort */
	CU(cudaMemcpyAsync(e->d.rp, e->h_rp, sizeof(ppi_rparams) * e->nrep, cudaMemcpyHostToDevice, e->stream));
	return PP_OK;
}

int pp_gpu_set_persistent(pp_engine *e, int enable) {
	if(e == NULL) return PP_ERR_ARG;
	enable = enable ? 1 : 0;
	if(enable == e->d.persist) return PP_OK;
	e->d.persist = enable;
	drop_graphs(e); /* the launches' arguments changed */
	return PP_OK;
}

int pp_gpu_set_barrier_test(pp_engine *e, long long limit_cycles, int unreachable) {
	if(e == NULL || limit_cycles < 0 || unreachable < 0 || unreachable > 1) return PP_ERR_ARG;
	e->d.bar_limit = limit_cycles;
	e->d.bar_extra = unreachable;
	drop_graphs(e);
	return PP_OK;
}

int pp_gpu_set_graphs(pp_engine *e, int enable) {
	if(e == NULL) return PP_ERR_ARG;
	/* GC / SUS exchanges and AVB batches are launched from the host between re-sort periods, which a
	 * captured period would skip */
	if(enable && (is_exchange(e) || e->any_avb || e->any_vmmc))
		return set_err(e, PP_ERR_ARG, "engines with insertions and removals, AVB or VMMC moves launch their kernels one by one (no graphs)");
	e->graphs_on = enable ? 1 : 0;
	if(!enable) drop_graphs(e);
	return PP_OK;
}

/* GC / SUS: the insertion and removal attempts of the coming re-sort period -- the reference makes
 * N_max x 0.01 per MC step on average (MC.c:33-35) -- then the new particle count for the launches that
 * follow (the re-sort places the particles in slots 0 .. N-1 into the cells) */
static int exchange_step(pp_engine *e) {
	const pp_params *p = e->prm;
	int per = (int) floor(0.01 * p->n_max + 0.5);
	if(per < 1) per = 1;
	long long nl = 0;
	CK(ppi_exchange(&e->d, e->epoch, per * e->resort_every, e->stream, &nl));
	e->launches += nl;
	int rc = read_states(e);
	if(rc != PP_OK) return rc;
	const int n = e->h_rs[0].n_live;
	e->N[0] = n;
	e->h_rp[0].N = n;
	e->d.ntot = n;
	return PP_OK;
}

int pp_gpu_sus_histogram(pp_engine *e, long long *hist, int reset) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(!is_exchange(e) || e->prm[0].ensemble != PP_SUS || e->d.sus_hist == NULL) return set_err(e, PP_ERR_ARG, "not an SUS engine");
	const int nb = e->prm[0].n_max - e->prm[0].n_min + 1;
	if(hist) {
		unsigned long long *tmp = malloc(sizeof(unsigned long long) * (size_t) nb);
		HOST_OK(tmp);
		cudaError_t c = cudaMemcpyAsync(tmp, e->d.sus_hist, sizeof(unsigned long long) * (size_t) nb, cudaMemcpyDeviceToHost, e->stream);
		if(c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
		for(int k = 0; k < nb && c == cudaSuccess; k++) hist[k] = (long long) tmp[k];
		free(tmp);
		if(c != cudaSuccess) return set_err(e, PP_ERR_CUDA, "SUS histogram copy: %s", cudaGetErrorString(c));
	}
	if(reset) CU(cudaMemsetAsync(e->d.sus_hist, 0, sizeof(unsigned long long) * (size_t) nb, e->stream));
	return PP_OK;
}

int pp_gpu_sweeps(pp_engine *e, long long n) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(n < 0) return set_err(e, PP_ERR_ARG, "negative sweep count");
	for(long long k = 0; k < n; k++) {
		/* whole re-sort periods from a captured graph (not while per-group event timing is on) */
		if(e->graphs_on && !e->graphs_broken && !e->timing && e->rounds_per_sweep == 1 && e->round_counter % e->resort_every == 0 && n - k >= e->resort_every) {
			rc = replay_period(e);
			if(rc == PP_OK) {
				k += e->resort_every - 1;
				continue;
			}
			if(rc != GRAPH_UNAVAILABLE) return rc;
			e->graphs_broken = 1;
		}
		long long s = e->sweep_counter++;
		int ev;
		if(e->any_vmmc) { /* every attempt a VMMC move (vmmc.c:258-483): N of them, then a re-sort for the passes that follow */
			long long nl = 0;
			if((rc = ev_begin(e, 1, &ev)) != PP_OK) return rc;
			CK(ppi_vmmc(&e->d, s, 1, e->stream, &nl));
			if((rc = ev_end(e, ev)) != PP_OK) return rc;
			e->launches += nl;
			if((rc = ev_begin(e, 0, &ev)) != PP_OK) return rc;
			if((rc = do_resort(e)) != PP_OK) return rc;
			if((rc = ev_end(e, ev)) != PP_OK) return rc;
			e->round_counter++;
		}
		for(int rr = 0; rr < (e->any_vmmc ? 0 : e->rounds_per_sweep); rr++) {
			if(e->round_counter % e->resort_every == 0) {
				if(is_exchange(e) && (rc = exchange_step(e)) != PP_OK) return rc;
				if(e->any_avb) { /* the AVB moves of the coming re-sort period (avb.c:77-186) */
					long long nl = 0;
					CK(ppi_avb(&e->d, e->epoch, e->resort_every, e->stream, &nl));
					e->launches += nl;
				}
				if((rc = ev_begin(e, 0, &ev)) != PP_OK) return rc;
				if((rc = do_resort(e)) != PP_OK) return rc;
				if((rc = ev_end(e, ev)) != PP_OK) return rc;
			}
			long long nl = 0;
			int colours[8];
			colour_order(e->round_counter, colours);
			if((rc = ev_begin(e, 1, &ev)) != PP_OK) return rc;
			if(e->proposal == PP_PROPOSAL_LEARNED) {
				CK(ppi_round_learned(&e->d, e->round_counter, colours, e->any_audit, e->stream, &nl));
				e->nl_valid = 0; /* learned moves reach farther than the lists' radius */
			}
			else CK(ppi_round(&e->d, e->round_counter, colours, e->any_audit, e->nl_valid, e->stream, &nl));
			if((rc = ev_end(e, ev)) != PP_OK) return rc;
			e->round_counter++;
			e->launches += nl;
		}
		if(e->any_npt || e->any_lx) { /* the sweep's NPT volume move or NVT box-shape move */
			long long nl = 0;
			if((rc = ev_begin(e, 2, &ev)) != PP_OK) return rc;
			CK(ppi_volume(&e->d, s, e->nl_valid && e->nl_all, e->stream, &nl));
			if(e->proposal == PP_PROPOSAL_LEARNED) CK(ppi_canon(&e->d, e->stream, &nl)); /* positions and box may have changed */
			if((rc = ev_end(e, ev)) != PP_OK) return rc;
			e->launches += nl;
		}
	}
	return PP_OK;
}

int pp_gpu_time_sweeps(pp_engine *e, long long n, double *ms) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	cudaEvent_t a, b;
	CU(cudaEventCreate(&a));
	CU(cudaEventCreate(&b));
	CU(cudaEventRecord(a, e->stream));
	rc = pp_gpu_sweeps(e, n);
	if(rc != PP_OK) return rc;
	CU(cudaEventRecord(b, e->stream));
	CU(cudaEventSynchronize(b));
	float t = 0.f;
	CU(cudaEventElapsedTime(&t, a, b));
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if(ms) *ms = t;
	return read_states(e);
}

int pp_gpu_sync(pp_engine *e) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	CU(cudaStreamSynchronize(e->stream));
	CU(cudaGetLastError());
	return read_states(e);
}

int pp_gpu_get_energy(pp_engine *e, int r, double *E) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep || E == NULL) return set_err(e, PP_ERR_ARG, "bad replica");
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	*E = -(double) e->h_rs[r].bonds;
	return PP_OK;
}

int pp_gpu_box(pp_engine *e, int r, double box[3]) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep || box == NULL) return set_err(e, PP_ERR_ARG, "bad replica or box pointer");
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	memcpy(box, e->h_rs[r].box, sizeof(double) * 3);
	return PP_OK;
}

int pp_gpu_energy(pp_engine *e, int r, double *E, int *overlap) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep) return set_err(e, PP_ERR_ARG, "bad replica");
	rc = run_energy(e, PPI_EN_BONDS);
	if(rc != PP_OK) return rc;
	if(E) *E = -0.5 * (double) e->h_rs[r].vol_bonds;
	if(overlap) *overlap = e->h_rs[r].vol_overlap;
	return PP_OK;
}

int pp_gpu_orthonormalise(pp_engine *e, int r) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep) return set_err(e, PP_ERR_ARG, "bad replica");
	long long nl = 0;
	ppi_rparams *rp = e->h_rp + r;
	CK(ppi_gram_schmidt(&e->d, rp->p0, rp->N, e->stream, &nl));
	e->launches += nl;
	/* the FP32 working records are rebuilt from the re-orthonormalised FP64 state */
	rc = do_resort(e);
	if(rc != PP_OK) return rc;
	e->round_counter += e->resort_every - e->round_counter % e->resort_every; /* start a fresh epoch */
	CU(cudaStreamSynchronize(e->stream));
	return PP_OK;
}

int pp_gpu_check_energy(pp_engine *e, int r) {
	double E;
	int ov;
	int rc = pp_gpu_energy(e, r, &E, &ov);
	if(rc != PP_OK) return rc;
	double tracked = -(double) e->h_rs[r].bonds;
	rc = pp_gpu_orthonormalise(e, r);
	if(rc != PP_OK) return rc;
	if(ov) return set_err(e, PP_ERR_OVERLAP, "Computing energy from scratch resulted in an overlap, aborting");
	if(fabs(tracked) > 1e-5 && fabs((E - tracked) / tracked) > 1e-5)
		return set_err(e, PP_ERR_DRIFT, "Energy check failed, old energy = %lf, new energy = %lf", tracked, E);
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	e->h_rs[r].bonds = (long long) llround(-E);
	return write_states(e);
}

int pp_gpu_counters(pp_engine *e, int r, pp_counters *out, int reset) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep) return set_err(e, PP_ERR_ARG, "bad replica");
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	if(out) {
		for(int k = 0; k < PP_N_MOVES; k++) {
			out->tries[k] = (long long) e->h_rs[r].tries[k];
			out->accepted[k] = (long long) e->h_rs[r].accepted[k];
		}
	}
	if(reset) {
		memset(e->h_rs[r].tries, 0, sizeof(e->h_rs[r].tries));
		memset(e->h_rs[r].accepted, 0, sizeof(e->h_rs[r].accepted));
		rc = write_states(e);
		if(rc != PP_OK) return rc;
		CU(cudaStreamSynchronize(e->stream));
	}
	return PP_OK;
}

int pp_gpu_guard_stats(pp_engine *e, pp_guard_stats *out, int reset) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	pp_guard_stats g;
	memset(&g, 0, sizeof(g));
	for(int r = 0; r < e->nrep; r++) {
		ppi_rstate *s = e->h_rs + r;
		g.pairs += (long long) s->pairs;
		g.fallbacks += (long long) s->fallbacks;
		g.mismatches += (long long) s->mismatches;
		g.nl_overflows += (long long) s->nl_overflow;
		float a, b;
		memcpy(&a, &s->max_err_r2_bits, 4);
		memcpy(&b, &s->max_err_cos_bits, 4);
		if(a > g.max_err_r2) g.max_err_r2 = a;
		if(b > g.max_err_cos) g.max_err_cos = b;
		if(reset) {
			s->pairs = s->fallbacks = s->mismatches = 0;
			s->max_err_r2_bits = s->max_err_cos_bits = 0;
			s->nl_overflow = 0;
		}
	}
	if(out) *out = g;
	if(reset) {
		rc = write_states(e);
		if(rc != PP_OK) return rc;
		CU(cudaStreamSynchronize(e->stream));
	}
	return PP_OK;
}

int pp_gpu_download_replica(pp_engine *e, int r, double *rr, double *RR, double box[3]) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep) return set_err(e, PP_ERR_ARG, "bad replica");
	rc = read_states(e);
	if(rc != PP_OK) return rc;
	ppi_rparams *rp = e->h_rp + r;
	int N = rp->N;
	long long nl = 0;
	CK(ppi_export(&e->d, rp->p0, N, e->stream, &nl)); /* x y z R = R0 . Q(q), 12 doubles per slot */
	e->launches += nl;
	CU(cudaMemcpyAsync(e->pin_rec, e->d.tmp_rec, sizeof(double) * 12 * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaMemcpyAsync(e->pin_id, e->d.id + rp->p0, sizeof(int) * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	for(int k = 0; k < N; k++) {
		int i = e->pin_id[k];
		if(i < 0 || i >= N) return set_err(e, PP_ERR_STATE, "corrupt particle ids");
		const double *src = e->pin_rec + (size_t) k * 12;
		if(rr) memcpy(rr + 3 * (size_t) i, src, 3 * sizeof(double));
		if(RR) memcpy(RR + 9 * (size_t) i, src + 3, 9 * sizeof(double));
	}
	if(box) memcpy(box, e->h_rs[r].box, sizeof(double) * 3);
	return PP_OK;
}

int pp_gpu_download(pp_engine *e, double *r, double *R, double box[3]) { return pp_gpu_download_replica(e, 0, r, R, box); }

static int fetch_counts(pp_engine *e, int r, int mode) {
	int rc = run_energy(e, mode);
	if(rc != PP_OK) return rc;
	ppi_rparams *rp = e->h_rp + r;
	int N = rp->N;
	CU(cudaMemcpyAsync(e->pin_i2, e->d.out_bonds + rp->p0, sizeof(int) * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaMemcpyAsync(e->pin_id, e->d.id + rp->p0, sizeof(int) * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	return PP_OK;
}

int pp_gpu_bonds(pp_engine *e, int r, int *n_bonds, int *n_overlaps) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep) return set_err(e, PP_ERR_ARG, "bad replica");
	rc = fetch_counts(e, r, PPI_EN_BONDS);
	if(rc != PP_OK) return rc;
	ppi_rparams *rp = e->h_rp + r;
	int N = rp->N;
	CU(cudaMemcpyAsync(e->pin_i1, e->d.out_overlaps + rp->p0, sizeof(int) * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	for(int k = 0; k < N; k++) {
		int i = e->pin_id[k];
		if(i < 0 || i >= N) return set_err(e, PP_ERR_STATE, "corrupt particle ids");
		if(n_bonds) n_bonds[i] = e->pin_i2[k];
		if(n_overlaps) n_overlaps[i] = e->pin_i1[k];
	}
	return PP_OK;
}

static int cmp_int(const void *a, const void *b) {
	int x = *(const int *) a, y = *(const int *) b;
	return (x > y) - (x < y);
}

int pp_gpu_bond_lists(pp_engine *e, int r, int *offsets, int *partners, int cap) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep || offsets == NULL) return set_err(e, PP_ERR_ARG, "bad arguments");
	rc = fetch_counts(e, r, PPI_EN_PARTNERS);
	if(rc != PP_OK) return rc;
	ppi_rparams *rp = e->h_rp + r;
	int N = rp->N;
	CU(cudaMemcpyAsync(e->pin_i1, e->d.out_partners + (size_t) rp->p0 * PPI_MAX_PARTNERS, sizeof(int) * PPI_MAX_PARTNERS * N, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	/* counts in upload order, then offsets, then the lists */
	int *cnt = calloc(N > 0 ? N : 1, sizeof(int));
	int *where = calloc(N > 0 ? N : 1, sizeof(int));
	if(cnt == NULL || where == NULL) {
		free(cnt);
		free(where);
		return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	}
	for(int k = 0; k < N; k++) {
		int i = e->pin_id[k];
		if(i < 0 || i >= N) {
			free(cnt);
			free(where);
			return set_err(e, PP_ERR_STATE, "corrupt particle ids");
		}
		cnt[i] = e->pin_i2[k];
		where[i] = k;
		if(cnt[i] > PPI_MAX_PARTNERS) {
			free(cnt);
			free(where);
			return set_err(e, PP_ERR_CAPACITY, "particle %d has more than %d bonds", i, PPI_MAX_PARTNERS);
		}
	}
	int total = 0;
	for(int i = 0; i < N; i++) {
		offsets[i] = total;
		total += cnt[i];
	}
	offsets[N] = total;
	if(total > cap || (total > 0 && partners == NULL)) {
		free(cnt);
		free(where);
		return set_err(e, PP_ERR_CAPACITY, "partner buffer holds %d entries, %d needed", cap, total);
	}
	for(int i = 0; i < N; i++) {
		memcpy(partners + offsets[i], e->pin_i1 + (size_t) where[i] * PPI_MAX_PARTNERS, sizeof(int) * cnt[i]);
		qsort(partners + offsets[i], cnt[i], sizeof(int), cmp_int);
	}
	free(cnt);
	free(where);
	return total;
}

/* ------------------------------------------------------------------------------------------------ */
/* .rrr format                                                                                      */
/* ------------------------------------------------------------------------------------------------ */
int pp_rrr_header(const char *path, long long *step, int *N, double box[3]) {
	FILE *f = fopen(path, "r");
	if(f == NULL) return PP_ERR_IO;
	long long st;
	int n;
	double b[3];
	int res = fscanf(f, "%lld %d %lf %lf %lf", &st, &n, b, b + 1, b + 2);
	fclose(f);
	if(res != 5 || n < 0) return PP_ERR_IO;
	if(step) *step = st;
	if(N) *N = n;
	if(box) memcpy(box, b, sizeof(b));
	return PP_OK;
}

static void set_msg(char *err, int len, const char *fmt, ...) {
	if(err == NULL || len <= 0) return;
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(err, len, fmt, ap);
	va_end(ap);
}

/* system.c:77-245: header "%*d %d %lf %lf %lf", then per particle: row 0 via fgets + sscanf, row 1 and the
 * position via fscanf; rows normalised, row 2 = row0 x row1, gram_schmidt. */
int pp_rrr_read(const char *path, int N, double *r, double *R, double box[3], char *err, int err_len) {
	if(path == NULL || N < 0 || (N > 0 && (r == NULL || R == NULL))) {
		set_msg(err, err_len, "pp_rrr_read: bad arguments");
		return PP_ERR_ARG;
	}
	FILE *f = fopen(path, "r");
	if(f == NULL) {
		set_msg(err, err_len, "Initial_conditions_file '%s' is not readable", path);
		return PP_ERR_IO;
	}
	int n;
	double b[3];
	if(fscanf(f, "%*d %d %lf %lf %lf\n", &n, b, b + 1, b + 2) != 4) {
		fclose(f);
		set_msg(err, err_len, "The initial configuration file '%s' is empty or its headers are malformed", path);
		return PP_ERR_IO;
	}
	if(n != N) {
		fclose(f);
		set_msg(err, err_len, "header of '%s' announces %d particles, caller expected %d", path, n, N);
		return PP_ERR_IO;
	}
	if(box) memcpy(box, b, sizeof(b));
	int i = 0;
	double p1[3] = { 0., 0., 0. }, p2[3] = { 0., 0., 0. }, p3[3], rp[3] = { 0., 0., 0. };
	char line[512];
	char *sr = fgets(line, sizeof(line), f);
	while(sr != NULL) {
		/* the reference does not check these scans either: a short record keeps the previous values */
		int got = sscanf(line, "%lf %lf %lf\n", p1, p1 + 1, p1 + 2);
		got += fscanf(f, "%lf %lf %lf\n", p2, p2 + 1, p2 + 2);
		got += fscanf(f, "%lf %lf %lf\n", rp, rp + 1, rp + 2);
		(void) got;
		if(i >= N) { /* records beyond the header's count are only counted, for the message below */
			i++;
			sr = fgets(line, sizeof(line), f);
			continue;
		}
		h_normalize(p1);
		h_normalize(p2);
		h_cross(p1, p2, p3);
		double *Ri = R + 9 * (size_t) i;
		memcpy(Ri, p1, sizeof(p1));
		memcpy(Ri + 3, p2, sizeof(p2));
		memcpy(Ri + 6, p3, sizeof(p3));
		h_gram_schmidt(Ri, Ri + 3, Ri + 6);
		memcpy(r + 3 * (size_t) i, rp, sizeof(rp));
		i++;
		sr = fgets(line, sizeof(line), f);
	}
	fclose(f);
	if(i != N) {
		set_msg(err, err_len, "Number of particles found in configuration (%d) is different from the value found in the header (%d)", i, N);
		return PP_ERR_IO;
	}
	return PP_OK;
}

int pp_rrr_write(const char *path, long long step, int N, const double *r, const double *R, const double box[3]) {
	if(path == NULL || box == NULL || N < 0 || (N > 0 && (r == NULL || R == NULL))) return PP_ERR_ARG;
	FILE *out = fopen(path, "w");
	if(out == NULL) return PP_ERR_IO;
	fprintf(out, "%lld %d %.12lf %.12lf %.12lf\n", step, N, box[0], box[1], box[2]); /* output.c:306 */
	for(int i = 0; i < N; i++) {
		const double *Ri = R + 9 * (size_t) i, *ri = r + 3 * (size_t) i;
		fprintf(out, "%lf %lf %lf\n", Ri[0], Ri[1], Ri[2]);
		fprintf(out, "%lf %lf %lf\n", Ri[3], Ri[4], Ri[5]);
		fprintf(out, "%.12lf %.12lf %.12lf\n", ri[0], ri[1], ri[2]);
	}
	const int bad = ferror(out);
	if(fclose(out) != 0 || bad) return PP_ERR_IO; /* a short write (full disk) is not a saved configuration */
	return PP_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* generator (generator.c)                                                                          */
/* ------------------------------------------------------------------------------------------------ */
typedef struct {
	unsigned long long X;
} g_rng;

static double g_drand(g_rng *g) { /* POSIX drand48 recurrence */
	g->X = (0x5DEECE66DULL * g->X + 0xBULL) & 0xFFFFFFFFFFFFULL;
	return (double) g->X * 0x1p-48;
}

static void g_sphere(g_rng *g, double *res) { /* random_vector_on_sphere, utils.c:115-131 */
	double a, b, s;
	do {
		a = 1. - 2. * g_drand(g);
		b = 1. - 2. * g_drand(g);
		s = a * a + b * b;
	} while(s >= 1.);
	double h = 2. * sqrt(1. - s);
	res[0] = a * h;
	res[1] = b * h;
	res[2] = 1. - 2. * s;
}

static double g_det(const double *m) { /* determinant, utils.c:78-89 */
	double det = 0.;
	det += m[0] * m[4] * m[8];
	det += m[1] * m[5] * m[6];
	det += m[2] * m[3] * m[7];
	det -= m[2] * m[4] * m[6];
	det -= m[0] * m[5] * m[7];
	det -= m[1] * m[3] * m[8];
	return det;
}

static void g_orientation(g_rng *g, double *R) { /* random_orientation, utils.c:133-169 */
	double x[3], y[3], z[3];
	g_sphere(g, x);
	g_sphere(g, y);
	g_sphere(g, z);
	h_gram_schmidt(x, y, z);
	memcpy(R, z, sizeof(z));
	memcpy(R + 3, x, sizeof(x));
	memcpy(R + 6, y, sizeof(y));
	if(g_det(R) < 0) {
		memcpy(R, x, sizeof(x));
		memcpy(R + 3, z, sizeof(z));
	}
}

static double round_text(const char *fmt, double v) {
	char buf[64];
	snprintf(buf, sizeof(buf), fmt, v);
	return strtod(buf, NULL);
}

int pp_generate(int N, double density, int seed, int round_like_file, double *r, double *R, double box[3]) {
	if(N < 0 || !(density > 0.) || density > 0.7 || r == NULL || R == NULL || box == NULL) return PP_ERR_ARG; /* generator.c:99-102 */
	double L = pow(N / density, 1. / 3.); /* generator.c:103-105 */
	g_rng g = { ((unsigned long long) (unsigned int) seed << 16) | 0x330EULL };
	/* cells of edge >= 1 (cells_init with rcut = 1, cells.c:17-37) */
	int ns = (int) floor(L / 1.);
	if(ns < 3) ns = 3;
	long long nc = (long long) ns * ns * ns;
	int *head = malloc(sizeof(int) * nc);
	int *next = malloc(sizeof(int) * (N > 0 ? N : 1));
	if(head == NULL || next == NULL) {
		free(head);
		free(next);
		return PP_ERR_CAPACITY;
	}
	for(long long c = 0; c < nc; c++) head[c] = -1;
	double bx[3] = { L, L, L };
	int inserted = 0;
	while(inserted < N) { /* make_initial_conf, generator.c:43-68 */
		double p[3] = { g_drand(&g) * L, g_drand(&g) * L, g_drand(&g) * L };
		int ind[3];
		for(int k = 0; k < 3; k++) ind[k] = (int) ((p[k] / bx[k] - floor(p[k] / bx[k])) * (1. - DBL_EPSILON) * ns);
		int over = 0;
		for(int j = -1; j < 2 && !over; j++)
			for(int k = -1; k < 2 && !over; k++)
				for(int l = -1; l < 2 && !over; l++) {
					int cx = (ind[0] + j + ns) % ns, cy = (ind[1] + k + ns) % ns, cz = (ind[2] + l + ns) % ns;
					int q = head[((long long) cx * ns + cy) * ns + cz];
					while(q != -1) {
						const double *rq = r + 3 * (size_t) q;
						double d[3] = { rq[0] - p[0], rq[1] - p[1], rq[2] - p[2] };
						for(int a = 0; a < 3; a++) d[a] -= bx[a] * rint(d[a] / bx[a]);
						if(H_SCALAR(d, d) < 1.) {
							over = 1;
							break;
						}
						q = next[q];
					}
				}
		if(over) continue;
		g_orientation(&g, R + 9 * (size_t) inserted);
		memcpy(r + 3 * (size_t) inserted, p, sizeof(p));
		int c = (ind[0] * ns + ind[1]) * ns + ind[2];
		next[inserted] = head[c];
		head[c] = inserted;
		inserted++;
	}
	free(head);
	free(next);
	box[0] = box[1] = box[2] = L;
	if(round_like_file) {
		/* what writing generated.rrr (generator.c:70-82) and reading it back (system.c:80-243) gives */
		double Lr = round_text("%lf", L);
		box[0] = box[1] = box[2] = Lr;
		for(int i = 0; i < N; i++) {
			double *Ri = R + 9 * (size_t) i, *ri = r + 3 * (size_t) i;
			double p1[3], p2[3], p3[3];
			for(int k = 0; k < 3; k++) {
				p1[k] = round_text("%lf", Ri[k]);
				p2[k] = round_text("%lf", Ri[3 + k]);
				ri[k] = round_text("%.12lf", ri[k]);
			}
			h_normalize(p1);
			h_normalize(p2);
			h_cross(p1, p2, p3);
			memcpy(Ri, p1, sizeof(p1));
			memcpy(Ri + 3, p2, sizeof(p2));
			memcpy(Ri + 6, p3, sizeof(p3));
			h_gram_schmidt(Ri, Ri + 3, Ri + 6);
		}
	}
	return PP_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* learned proposal                                                                                 */
/* ------------------------------------------------------------------------------------------------ */
void pp_default_learned_params(pp_learned_params *p) {
	memset(p, 0, sizeof(*p));
	const double sd[PP_MIX] = { 1., 4., 8., 8. }, st[PP_MIX] = { 1., 4., 8., 25. };
	for(int k = 0; k < PP_MIX; k++) {
		p->scale_disp[k] = sd[k];
		p->scale_theta[k] = st[k];
	}
	p->floor = 0.1;
	p->entropy = 0.01;
	p->kappa = 1.;
	p->jump = 1e-9;
	p->draws = 4;
	p->seed = 12345;
}

static uint64_t splitmix64(uint64_t *s) {
	uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

static double u01_sm(uint64_t *s) { return (double) (splitmix64(s) >> 11) * 0x1p-53; }

/* layout-sized buffers (canonical images, features); valid after the layout exists */
static int ensure_learn_layout(pp_engine *e) {
	if(!e->committed) return set_err(e, PP_ERR_STATE, "no configuration uploaded for every replica");
	if(!e->d.simg || !e->d.feat) drop_graphs(e); /* captured launches hold the device pointers by value */
	size_t n1 = e->ntot_alloc > 0 ? (size_t) e->ntot_alloc : 1;
	if(!e->d.simg) CU(cudaMalloc((void **) &e->d.simg, sizeof(float) * 16 * n1));
	if(!e->d.feat) CU(cudaMalloc((void **) &e->d.feat, sizeof(float) * PP_MLP_IN * n1));
	return PP_OK;
}

static int learn_check(pp_engine *e) {
	if(e == NULL) return PP_ERR_ARG;
	if(!e->learn_ready) return set_err(e, PP_ERR_STATE, "learned proposal not initialised (pp_gpu_learned_init)");
	return PP_OK;
}

int pp_gpu_learned_init(pp_engine *e, const pp_learned_params *p) {
	if(e == NULL || p == NULL) return PP_ERR_ARG;
	if(p->scale_disp[0] != 1. || p->scale_theta[0] != 1.) return set_err(e, PP_ERR_ARG, "component 0 is the plain move: its scales must be 1");
	for(int k = 0; k < PP_MIX; k++)
		if(!(p->scale_disp[k] > 0.) || !(p->scale_theta[k] > 0.) || p->scale_disp[k] > 1e3 || p->scale_theta[k] > 1e3)
			return set_err(e, PP_ERR_ARG, "component scales must lie in (0, 1000]");
	if(!(p->floor > 0. && p->floor <= 1.)) return set_err(e, PP_ERR_ARG, "floor must lie in (0, 1]");
	if(!(p->entropy >= 0.) || !(p->kappa >= 0.) || !(p->jump >= 0.)) return set_err(e, PP_ERR_ARG, "entropy, kappa and jump must be >= 0");
	if(p->draws < 1 || p->draws > 64) return set_err(e, PP_ERR_ARG, "draws must lie in [1, 64]");
	e->lprm = *p;
	for(int k = 0; k < PP_MIX; k++) {
		e->h_learn.sdisp[k] = (float) p->scale_disp[k];
		e->h_learn.stheta[k] = (float) p->scale_theta[k];
	}
	e->h_learn.floor0 = (float) p->floor;
	e->h_learn.kappa = (float) p->kappa;
	e->h_learn.jump = (float) p->jump;
	e->h_learn.draws = p->draws;
	if(!e->learn_ready) {
		CU(cudaMalloc((void **) &e->l_P, sizeof(float) * PP_MLP_NPARAMS));
		CU(cudaMalloc((void **) &e->l_m1, sizeof(float) * PP_MLP_NPARAMS));
		CU(cudaMalloc((void **) &e->l_m2, sizeof(float) * PP_MLP_NPARAMS));
		CU(cudaMalloc((void **) &e->l_grad, sizeof(float) * PP_MLP_NPARAMS));
		CU(cudaMalloc((void **) &e->l_img, 32768));
		CU(cudaMalloc((void **) &e->l_learn, sizeof(ppi_learn)));
		CU(cudaMalloc((void **) &e->l_rep, sizeof(ppi_lrep) * (size_t) e->nrep));
		CU(cudaMalloc((void **) &e->l_stats, sizeof(unsigned long long) * 2 * PP_MIX));
		CU(cudaMalloc((void **) &e->l_err, sizeof(int)));
		CU(cudaMalloc((void **) &e->l_obj, sizeof(double)));
		e->learn_ready = 1;
	}
	drop_graphs(e);
	e->d.mlp_img = e->l_img;
	e->d.learn = e->l_learn;
	e->d.lrep = e->l_rep;
	e->d.lstats = e->l_stats;
	{ /* per replica tables: the component edges and angles as the kernels' FP32 values, their densities */
		ppi_lrep *M = calloc((size_t) e->nrep, sizeof(ppi_lrep));
		if(!M) return set_err(e, PP_ERR_CAPACITY, "out of host memory");
		for(int r = 0; r < e->nrep; r++) {
			const float dm = (float) e->prm[r].disp_max, tm = (float) e->prm[r].theta_max;
			for(int k = 0; k < PP_MIX; k++) {
				const float a = k == 0 ? dm : dm * e->h_learn.sdisp[k];
				float t = k == 0 ? tm : tm * e->h_learn.stheta[k];
				if(t > 3.1415925f) t = 3.1415925f; /* rotation angles stay below pi */
				M[r].a[k] = a;
				M[r].t[k] = t;
				M[r].v[k] = 1.0 / ((double) a * (double) a * (double) a * (double) t);
			}
			for(int k = -PPI_LEXP; k <= PPI_LEXP; k++) M[r].expk[k + PPI_LEXP] = exp(-(double) k / e->prm[r].temperature);
			if(!(M[r].a[0] > 0.f) || !(M[r].t[0] > 0.f)) {
				free(M);
				return set_err(e, PP_ERR_ARG, "replica %d: the learned proposal needs Disp_max > 0 and Theta_max > 0", r);
			}
		}
		cudaError_t c = cudaMemcpy(e->l_rep, M, sizeof(ppi_lrep) * (size_t) e->nrep, cudaMemcpyHostToDevice);
		free(M);
		if(c != cudaSuccess) return set_err(e, PP_ERR_CUDA, "mixture tables: %s", cudaGetErrorString(c));
	}
	e->d.lerr = e->l_err;
	CU(cudaMemcpyAsync(e->l_learn, &e->h_learn, sizeof(ppi_learn), cudaMemcpyHostToDevice, e->stream));
	CU(cudaMemsetAsync(e->l_stats, 0, sizeof(unsigned long long) * 2 * PP_MIX, e->stream));
	CU(cudaMemsetAsync(e->l_err, 0, sizeof(int), e->stream));
	/* initial weights: uniform fan-in hidden layers, zero biases and output layer (uniform mixture) */
	float *P = calloc(PP_MLP_NPARAMS, sizeof(float));
	if(!P) return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	uint64_t st = p->seed;
	const double a1 = sqrt(6.0 / PP_MLP_IN), a2 = sqrt(6.0 / PP_MLP_HIDDEN);
	for(int i = 0; i < PP_MLP_HIDDEN * PP_MLP_IN; i++) P[i] = (float) ((2. * u01_sm(&st) - 1.) * a1);
	const int w2 = PP_MLP_HIDDEN * PP_MLP_IN + PP_MLP_HIDDEN;
	for(int i = 0; i < PP_MLP_HIDDEN * PP_MLP_HIDDEN; i++) P[w2 + i] = (float) ((2. * u01_sm(&st) - 1.) * a2);
	int rc = pp_gpu_learned_set_weights(e, P);
	free(P);
	return rc;
}

int pp_gpu_learned_set_weights(pp_engine *e, const float *params) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	if(params == NULL) return set_err(e, PP_ERR_ARG, "null weights");
	for(int i = 0; i < PP_MLP_NPARAMS; i++)
		if(!isfinite(params[i])) return set_err(e, PP_ERR_ARG, "weight %d is not finite", i);
	CU(cudaMemcpyAsync(e->l_P, params, sizeof(float) * PP_MLP_NPARAMS, cudaMemcpyHostToDevice, e->stream));
	CU(cudaMemsetAsync(e->l_m1, 0, sizeof(float) * PP_MLP_NPARAMS, e->stream));
	CU(cudaMemsetAsync(e->l_m2, 0, sizeof(float) * PP_MLP_NPARAMS, e->stream));
	CU(cudaMemsetAsync(e->l_grad, 0, sizeof(float) * PP_MLP_NPARAMS, e->stream));
	e->adam_step = 0;
	CK(ppi_mlp_pack(e->l_P, e->l_img, e->stream));
	e->launches++;
	CU(cudaStreamSynchronize(e->stream));
	return PP_OK;
}

int pp_gpu_learned_get_weights(pp_engine *e, float *params) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	if(params == NULL) return set_err(e, PP_ERR_ARG, "null weights");
	CU(cudaMemcpyAsync(params, e->l_P, sizeof(float) * PP_MLP_NPARAMS, cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	return PP_OK;
}

int pp_gpu_set_proposal(pp_engine *e, int proposal) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(proposal != PP_PROPOSAL_PLAIN && is_exchange(e)) return set_err(e, PP_ERR_ARG, "the learned proposal is not available with insertions and removals");
	if(proposal != PP_PROPOSAL_PLAIN && (e->any_avb || e->any_vmmc)) return set_err(e, PP_ERR_ARG, "the learned proposal is not available with AVB or VMMC moves");
	if(proposal == PP_PROPOSAL_PLAIN) {
		e->proposal = proposal;
		return PP_OK;
	}
	if(proposal != PP_PROPOSAL_LEARNED) return set_err(e, PP_ERR_ARG, "unknown proposal %d", proposal);
	rc = learn_check(e);
	if(rc != PP_OK) return rc;
	rc = ensure_learn_layout(e);
	if(rc != PP_OK) return rc;
	long long nl = 0;
	CK(ppi_canon(&e->d, e->stream, &nl));
	e->launches += nl;
	e->proposal = proposal;
	return PP_OK;
}


/* grows the device sample buffer to hold at least n samples (existing samples kept) */
static int ensure_samples(pp_engine *e, long long n) {
	if(n <= e->d.sample_cap) return PP_OK;
	if(n > (1LL << 30)) return set_err(e, PP_ERR_CAPACITY, "too many training samples");
	long long cap = e->d.sample_cap > 0 ? 2LL * e->d.sample_cap : 1024;
	while(cap < n) cap *= 2;
	float *buf = NULL;
	CU(cudaMalloc((void **) &buf, sizeof(float) * PP_MLP_SAMPLE * (size_t) cap));
	if(e->n_samples > 0) CU(cudaMemcpyAsync(buf, e->d.samples, sizeof(float) * PP_MLP_SAMPLE * (size_t) e->n_samples, cudaMemcpyDeviceToDevice, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	if(e->d.samples) cudaFree(e->d.samples);
	e->d.samples = buf;
	e->d.sample_cap = (int) cap;
	return PP_OK;
}

int pp_gpu_learned_collect(pp_engine *e, int n_configs, int sweeps_between, int samples_per_config) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	rc = learn_check(e);
	if(rc != PP_OK) return rc;
	if(n_configs < 0 || sweeps_between < 0 || samples_per_config < 1) return set_err(e, PP_ERR_ARG, "bad collection arguments");
	rc = ensure_learn_layout(e);
	if(rc != PP_OK) return rc;
	rc = ensure_samples(e, e->n_samples + (long long) n_configs * samples_per_config);
	if(rc != PP_OK) return rc;
	const int saved = e->proposal;
	e->proposal = PP_PROPOSAL_PLAIN; /* the training configurations come from the plain move */
	for(int c = 0; c < n_configs; c++) {
		rc = pp_gpu_sweeps(e, sweeps_between);
		if(rc != PP_OK) break;
		long long nl = 0;
		int order[8];
		colour_order(e->collect_snap, order);
		if((rc = ppi_canon(&e->d, e->stream, &nl)) != 0 ||
				(rc = ppi_learn_collect(&e->d, e->collect_snap, order[0], (int) e->n_samples, samples_per_config, e->stream, &nl)) != 0) {
			rc = set_err(e, PP_ERR_CUDA, "sample collection: %s", cudaGetErrorString((cudaError_t) rc));
			break;
		}
		e->launches += nl;
		e->collect_snap++;
		e->n_samples += samples_per_config;
	}
	e->proposal = saved;
	if(rc != PP_OK) return rc;
	CU(cudaStreamSynchronize(e->stream));
	return read_states(e);
}

int pp_gpu_learned_samples(pp_engine *e, long long *count, float *out) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	if(count) *count = e->n_samples;
	if(out && e->n_samples > 0) {
		CU(cudaMemcpyAsync(out, e->d.samples, sizeof(float) * PP_MLP_SAMPLE * (size_t) e->n_samples, cudaMemcpyDeviceToHost, e->stream));
		CU(cudaStreamSynchronize(e->stream));
	}
	return PP_OK;
}

int pp_gpu_learned_clear_samples(pp_engine *e) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	e->n_samples = 0;
	return PP_OK;
}

int pp_gpu_learned_train(pp_engine *e, int epochs, int tiles_per_cta, double lr, double *objective) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	if(epochs < 0 || tiles_per_cta < 1 || tiles_per_cta > 64 || !(lr > 0.) || lr > 1.) return set_err(e, PP_ERR_ARG, "bad training arguments");
	if(e->n_samples == 0) return set_err(e, PP_ERR_STATE, "no training samples (pp_gpu_learned_collect)");
	const int ntiles = (int) ((e->n_samples + 127) / 128);
	if(e->l_tiles_cap < ntiles) {
		if(e->l_tiles) cudaFree(e->l_tiles);
		e->l_tiles = NULL;
		CU(cudaMalloc((void **) &e->l_tiles, sizeof(int) * (size_t) ntiles));
		e->l_tiles_cap = ntiles;
	}
	int *perm = malloc(sizeof(int) * (size_t) ntiles);
	if(!perm) return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	int ctas = ppi_sm_count();
	if(ctas * tiles_per_cta > ntiles) ctas = (ntiles + tiles_per_cta - 1) / tiles_per_cta;
	const int per_step = ctas * tiles_per_cta;
	double obj_sum = 0.;
	long long obj_n = 0;
	uint64_t st = e->lprm.seed ^ 0xA5A5A5A5DEADBEEFULL;
	for(int ep = 0; ep < epochs && rc == PP_OK; ep++) {
		for(int i = 0; i < ntiles; i++) perm[i] = i;
		for(int i = ntiles - 1; i > 0; i--) {
			int j = (int) (splitmix64(&st) % (uint64_t) (i + 1));
			int t = perm[i];
			perm[i] = perm[j];
			perm[j] = t;
		}
		if(cudaMemcpyAsync(e->l_tiles, perm, sizeof(int) * (size_t) ntiles, cudaMemcpyHostToDevice, e->stream) != cudaSuccess) {
			rc = set_err(e, PP_ERR_CUDA, "tile order upload failed");
			break;
		}
		const int last = ep == epochs - 1;
		if(last) cudaMemsetAsync(e->l_obj, 0, sizeof(double), e->stream);
		for(int s0 = 0; s0 < ntiles; s0 += per_step) {
			const int nt = ntiles - s0 < per_step ? ntiles - s0 : per_step;
			int c = ppi_mlp_train_step(e->l_img, e->d.samples, (int) e->n_samples, e->l_tiles + s0, nt, tiles_per_cta, (float) e->lprm.floor, (float) e->lprm.entropy,
					1.f / (float) (nt * 128), e->l_grad, e->l_obj, e->l_err, e->stream);
			if(c == 0) c = ppi_mlp_adam(e->l_P, e->l_grad, e->l_m1, e->l_m2, e->l_img, ++e->adam_step, (float) lr, e->stream);
			if(c != 0) {
				rc = set_err(e, PP_ERR_CUDA, "training step: %s", cudaGetErrorString((cudaError_t) c));
				break;
			}
			e->launches += 2;
		}
		/* the copy of perm must finish before the next epoch overwrites it */
		if(cudaStreamSynchronize(e->stream) != cudaSuccess) rc = set_err(e, PP_ERR_CUDA, "training failed");
		if(last) obj_n = e->n_samples;
	}
	free(perm);
	if(rc != PP_OK) return rc;
	CU(cudaMemcpyAsync(&obj_sum, e->l_obj, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
	int lerr = 0;
	CU(cudaMemcpyAsync(&lerr, e->l_err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	if(lerr) return set_err(e, PP_ERR_CUDA, "a tensor-core wait of the training step timed out");
	if(objective) *objective = obj_n > 0 ? obj_sum / (double) obj_n : 0.;
	return PP_OK;
}

int pp_gpu_learned_features(pp_engine *e, int r, float *features) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(r < 0 || r >= e->nrep || features == NULL) return set_err(e, PP_ERR_ARG, "bad arguments");
	rc = learn_check(e);
	if(rc != PP_OK) return rc;
	rc = ensure_learn_layout(e);
	if(rc != PP_OK) return rc;
	long long nl = 0;
	CK(ppi_canon(&e->d, e->stream, &nl));
	CK(ppi_learn_features(&e->d, e->stream, &nl));
	e->launches += nl;
	ppi_rparams *rp = e->h_rp + r;
	const int N = rp->N;
	float *tmp = malloc(sizeof(float) * PP_MLP_IN * (size_t) (N > 0 ? N : 1));
	if(!tmp) return set_err(e, PP_ERR_CAPACITY, "out of host memory");
	if(cudaMemcpyAsync(tmp, e->d.feat + (size_t) rp->p0 * PP_MLP_IN, sizeof(float) * PP_MLP_IN * (size_t) N, cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
			cudaMemcpyAsync(e->pin_id, e->d.id + rp->p0, sizeof(int) * N, cudaMemcpyDeviceToHost, e->stream) != cudaSuccess ||
			cudaStreamSynchronize(e->stream) != cudaSuccess) {
		free(tmp);
		return set_err(e, PP_ERR_CUDA, "feature download failed");
	}
	for(int k = 0; k < N; k++) {
		const int i = e->pin_id[k];
		if(i < 0 || i >= N) {
			free(tmp);
			return set_err(e, PP_ERR_STATE, "corrupt particle ids");
		}
		memcpy(features + (size_t) i * PP_MLP_IN, tmp + (size_t) k * PP_MLP_IN, sizeof(float) * PP_MLP_IN);
	}
	free(tmp);
	return PP_OK;
}

int pp_gpu_learned_stats(pp_engine *e, long long tries[PP_MIX], long long accepted[PP_MIX], int reset) {
	int rc = learn_check(e);
	if(rc != PP_OK) return rc;
	unsigned long long v[2 * PP_MIX];
	CU(cudaMemcpyAsync(v, e->l_stats, sizeof(v), cudaMemcpyDeviceToHost, e->stream));
	CU(cudaStreamSynchronize(e->stream));
	for(int k = 0; k < PP_MIX; k++) {
		if(tries) tries[k] = (long long) v[k];
		if(accepted) accepted[k] = (long long) v[PP_MIX + k];
	}
	if(reset) CU(cudaMemsetAsync(e->l_stats, 0, sizeof(v), e->stream));
	return PP_OK;
}

/* ------------------------------------------------------------------------------------------------ */
/* autotuner                                                                                        */
/* ------------------------------------------------------------------------------------------------ */
/* minimum cell edge of replica r for the engine's current period and scale (as derive_rparams) */
static double tuned_w_min(const pp_engine *e, int r) {
	const pp_params *p = e->prm + r;
	double wm = (1. + p->kf_delta) + 1e-5;
	if(p->ensemble == PP_NPT) wm /= exp(-0.5 * p->rescale_factor_max * (e->resort_every + 1));
	double lsmin, lsmax;
	lx_move_bounds(p, e->h_box[r], &lsmin, &lsmax);
	wm /= pow(lsmin, e->resort_every + 1);
	return wm * e->cell_scale;
}

/* installs a schedule; the next round re-sorts onto the new grid */
static int apply_schedule(pp_engine *e, int resort, int reorder, double scale, int lists) {
	drop_graphs(e);
	e->resort_every = resort;
	e->reorder_every = reorder;
	e->cell_scale = scale;
	e->nl_mode = lists;
	for(int r = 0; r < e->nrep; r++) e->h_rp[r].w_min = tuned_w_min(e, r);
	int rc = setup_nlists(e); /* the lists' radius covers one period of motion */
	if(rc != PP_OK) return rc;
	e->nl_valid = 0;
	e->graph_gen++;
	CU(cudaMemcpyAsync(e->d.rp, e->h_rp, sizeof(ppi_rparams) * e->nrep, cudaMemcpyHostToDevice, e->stream));
	e->round_counter += (resort - e->round_counter % resort) % resort;
	return PP_OK;
}

static long long total_tries(pp_engine *e) {
	long long t = 0;
	for(int r = 0; r < e->nrep; r++) t += (long long) e->h_rs[r].tries[PP_MOVE_ROTO_TRASL] + (long long) e->h_rs[r].tries[PP_MOVE_VOLUME];
	return t;
}

/* attempts per second of the installed schedule over `sweeps` sweeps after two warm-up sweeps */
static int time_schedule(pp_engine *e, int sweeps, double *aps) {
	int rc = pp_gpu_sweeps(e, 2);
	if(rc == PP_OK) rc = read_states(e);
	if(rc != PP_OK) return rc;
	const long long t0 = total_tries(e);
	double ms = 0.;
	rc = pp_gpu_time_sweeps(e, sweeps, &ms);
	if(rc != PP_OK) return rc;
	const long long t1 = total_tries(e);
	*aps = ms > 0. ? (double) (t1 - t0) / (ms * 1e-3) : 0.;
	return PP_OK;
}

int pp_gpu_autotune(pp_engine *e, int trial_sweeps, pp_tune_result *out) {
	int rc = ready(e);
	if(rc != PP_OK) return rc;
	if(trial_sweeps < 1 || trial_sweeps > 100000) return set_err(e, PP_ERR_ARG, "trial_sweeps must lie in [1, 100000]");
	if(is_exchange(e)) return set_err(e, PP_ERR_ARG, "the autotuner does not run GC or SUS engines (their particle count changes)");
	if(e->any_avb || e->any_vmmc) return set_err(e, PP_ERR_ARG, "the autotuner does not run AVB or VMMC engines");
	const int resorts[] = { 1, 2, 4, 8, 16 }, reorders[] = { 4, 16, 64 };
	const double scales[] = { 1.0, 1.2, 1.5 };
	const int r0 = e->resort_every, o0 = e->reorder_every, l0 = e->nl_mode;
	const double s0 = e->cell_scale;
	double base = 0.;
	if((rc = time_schedule(e, trial_sweeps, &base)) != PP_OK) return rc;
	int best_r = r0, best_o = o0, best_l = l0, tried = 1;
	double best_s = s0, best = base;
	for(int l = l0; l >= 0; l--) /* lists on and off when the caller allows them */
		for(int a = 0; a < 5; a++)
			for(int b = 0; b < 3; b++)
				for(int c = 0; c < 3; c++) {
					if(resorts[a] == r0 && reorders[b] == o0 && scales[c] == s0 && l == l0) continue;
					if((rc = apply_schedule(e, resorts[a], reorders[b], scales[c], l)) != PP_OK) return rc;
					double v = 0.;
					rc = time_schedule(e, trial_sweeps, &v);
					if(rc != PP_OK) { /* a schedule the boxes cannot hold: fall back to the best so far */
						apply_schedule(e, best_r, best_o, best_s, best_l);
						return rc;
					}
					tried++;
					if(v > best) {
						best = v;
						best_r = resorts[a];
						best_o = reorders[b];
						best_s = scales[c];
						best_l = l;
					}
				}
	if((rc = apply_schedule(e, best_r, best_o, best_s, best_l)) != PP_OK) return rc;
	if(out) {
		out->resort_every = best_r;
		out->reorder_every = best_o;
		out->cell_scale = best_s;
		out->attempts_per_s = best;
		out->baseline_attempts_per_s = base;
		out->n_tried = tried;
		out->neighbour_lists = best_l;
	}
	return PP_OK;
}
