/*
 * gpu_ensemble.c -- the reference-side binding of the GB300 engine: a new file a maintainer adds to the
 * PatchyParticles sources (beside MC.c), compiled against the reference's own headers and this
 * repository's include/ppgpu.h, linked with libppgpu.so. It stands in for the per-step ensemble hook
 * `do_ensemble` (defs.h:77-78), selected in MC_init (MC.c:85-131) and called from main.c:119, and for the
 * print/save synchronisation points of the main loop (main.c:82-104) and MC_check_energy (MC.c:766-784).
 */
#include "defs.h"
#include "avb.h"
#include "vmmc.h"
#include "cells.h"
#include "output.h"
#include "utils.h"
#include "ppgpu.h"        /* from this repository's include/ */
#include <stdlib.h>

extern avbmc *avbdata;  /* avb.c:11, set by AVBMC_init (MC_init runs before gpu_ensemble_init) */
extern vmmc_d *vmmcdata; /* vmmc.c:13, set by VMMC_init */

static pp_engine *G = NULL;

/* after system_init (system.c:58) and MC_init: copy the System to the device */
int gpu_ensemble_init(System *syst, Output *IO, int seed) {
	pp_params p;
	pp_default_params(&p);
	p.ensemble = syst->ensemble;            /* 0 (NVT), 1 (GC), 3 (SUS) or 5 (NPT) */
	p.temperature = syst->T;
	p.pressure = syst->P;
	p.disp_max = syst->disp_max;
	p.theta_max = syst->theta_max;
	p.rescale_factor_max = syst->rescale_factor_max;
	p.kf_delta = syst->kf_delta;
	p.kf_cosmax = syst->kf_cosmax;
	p.lx_move = syst->Lx_move;              /* NVT box-shape move (system.c:170-196) */
	p.lx_change_max = syst->Lx_change_max;
	p.lyz_min = syst->Lyz_min;
	p.lyz_max = syst->Lyz_max;
	p.seed = (uint64_t) seed;
	p.dynamics = syst->dynamics; /* 0, 1 (VMMC, vmmc.c:258-483) or 2 (AVB moves and roto-translations, avb.c:77-186) */
	if(syst->dynamics == AVBMC) p.avb_p = avbdata->avb_p;
	if(syst->dynamics == VMMC) {
		p.vmmc_max_cluster = vmmcdata->max_cluster;
		p.vmmc_max_move = vmmcdata->max_move;
	}
	if(syst->ensemble == GC || syst->ensemble == SUS) { /* system.c:90-103 */
		p.activity = syst->z;
		p.n_min = syst->N_min;
		p.n_max = syst->N_max;
	}
	if(pp_gpu_create(&p, &G) != PP_OK) output_exit(IO, "%s\n", pp_gpu_last_error(G));
	double *r = malloc(sizeof(double) * 3 * syst->N), *R = malloc(sizeof(double) * 9 * syst->N);
	for(int i = 0; i < syst->N; i++) {
		PatchyParticle *q = syst->particles + i;
		for(int k = 0; k < 3; k++) r[3 * i + k] = q->r[k];
		for(int k = 0; k < 9; k++) R[9 * i + k] = q->orientation[k / 3][k % 3];
	}
	int rc = pp_gpu_upload(G, syst->N, r, R, syst->box);
	free(r);
	free(R);
	if(rc == PP_ERR_OVERLAP) output_exit(IO, "Initial configuration contains an overlap, aborting\n");
	if(rc != PP_OK) output_exit(IO, "%s\n", pp_gpu_last_error(G));
	return 0;
}

/* the do_ensemble hook: one MC step, enqueued asynchronously */
void gpu_do_ensemble(System *syst, Output *IO) {
	if(pp_gpu_sweeps(G, 1) != PP_OK) output_exit(IO, "%s\n", pp_gpu_last_error(G));
}

/* before output_print / output_save read the System (main.c:82-104) */
void gpu_sync_system(System *syst, Output *IO) {
	/* GC / SUS: the particle count changes on the device; the reference's particle array holds N_max
	 * (system.c:199), and particles 0 .. N-1 are the live ones, as after its own MC_add_remove */
	double *r = malloc(sizeof(double) * 3 * syst->N_max), *R = malloc(sizeof(double) * 9 * syst->N_max);
	pp_counters c;
	if(pp_gpu_download(G, r, R, syst->box) != PP_OK || pp_gpu_get_energy(G, 0, &syst->energy) != PP_OK ||
			pp_gpu_counters(G, 0, &c, 1) != PP_OK)
		output_exit(IO, "%s\n", pp_gpu_last_error(G));
	syst->N = pp_gpu_num_particles(G, 0);
	if(syst->ensemble == SUS) { /* fold the device histogram into SUS_hist, which output_and_reset_sus prints */
		int nb = syst->N_max - syst->N_min + 1;
		llint *h = malloc(sizeof(llint) * nb);
		if(pp_gpu_sus_histogram(G, h, 1) != PP_OK) output_exit(IO, "%s\n", pp_gpu_last_error(G));
		for(int k = 0; k < nb; k++) syst->SUS_hist[k] += h[k];
		free(h);
	}
	for(int i = 0; i < syst->N; i++) {
		PatchyParticle *q = syst->particles + i;
		q->index = i;
		for(int k = 0; k < 3; k++) q->r[k] = r[3 * i + k];
		for(int k = 0; k < 9; k++) q->orientation[k / 3][k % 3] = R[9 * i + k];
		set_patches(syst, q); /* the reference's patch vectors follow the orientation (utils.c:20-23) */
	}
	syst->V = syst->box[0] * syst->box[1] * syst->box[2];
	/* the reference's cell lists follow the new positions (output_print_bonds walks them): a new grid where
	 * the box became too small for the old one, as MC_change_volume does (MC.c:480-485), then a refill */
	Cells *cl = syst->cells;
	if(syst->box[0] / cl->N_side[0] < syst->r_cut || syst->box[1] / cl->N_side[1] < syst->r_cut ||
			syst->box[2] / cl->N_side[2] < syst->r_cut) {
		cells_free(cl);
		cells_init(syst, IO, syst->r_cut);
	}
	else {
		for(int i = 0; i < cl->N; i++) cl->heads[i] = NULL;
	}
	cells_fill(syst);
	for(int k = 0; k < N_MOVES; k++) {
		syst->tries[k] += (int) c.tries[k];
		syst->accepted[k] += (int) c.accepted[k];
	}
	free(r);
	free(R);
}

/* MC_check_energy (MC.c:766-784) on the device */
void gpu_check_energy(System *syst, Output *IO) {
	int rc = pp_gpu_check_energy(G, 0);
	if(rc == PP_ERR_OVERLAP) output_exit(IO, "\nComputing energy from scratch resulted in an overlap, aborting\n");
	if(rc != PP_OK) output_exit(IO, "\n%s\n", pp_gpu_last_error(G));
	pp_gpu_get_energy(G, 0, &syst->energy);
}
