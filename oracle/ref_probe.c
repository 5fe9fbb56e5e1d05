/*
 * ref_probe.c -- test infrastructure. Linked by oracle/Makefile against the reference's own sources
 * (never against the product) to print, for one reference input file, what the reference's routines
 * say about every particle of the configuration it names:
 *
 *   line 1 : "N E_total overlap_any"           (E_total = 0.5 * sum_i MC_energy(i), main.c:55-64)
 *   then per particle i (0-based, file order):
 *            "i E_i overlap_i n_bond n_overlap : bonded partners... | overlapping partners..."
 *
 * E_i and overlap_i come from MC_energy (MC.c:272-309), which stops at the first overlap; the partner
 * lists come from a full walk over the same 27 cells calling MC_interact (MC.c:268-270), as
 * output_print_bonds does (output.c:213-268), without stopping at overlaps.
 */
#include "defs.h"
#include "MC.h"
#include "cells.h"
#include "output.h"
#include "parse_input.h"
#include "system.h"
#include "utils.h"

#include <stdio.h>
#include <stdlib.h>

static int cmp_int(const void *a, const void *b) {
	int x = *(const int *) a, y = *(const int *) b;
	return (x > y) - (x < y);
}

int main(int argc, char *argv[]) {
	if(argc < 2) {
		fprintf(stderr, "usage: %s input_file\n", argv[0]);
		return 1;
	}
	Output out;
	out.log = stderr;
	input_file input;
	loadInputFile(&input, argv[1]);
	if(input.state == ERROR) return 1;
	System syst;
	system_init(&input, &syst, &out);

	int N = syst.N;
	double *E = malloc(sizeof(double) * (N > 0 ? N : 1));
	int *ov = malloc(sizeof(int) * (N > 0 ? N : 1));
	double E_tot = 0.;
	int any = 0;
	for(int i = 0; i < N; i++) {
		E[i] = MC_energy(&syst, syst.particles + i);
		ov[i] = syst.overlap;
		if(ov[i]) any = 1;
		E_tot += E[i];
	}
	E_tot *= 0.5;
	printf("%d %.17g %d\n", N, E_tot, any);

	int *bonded = malloc(sizeof(int) * (N > 0 ? N : 1));
	int *overl = malloc(sizeof(int) * (N > 0 ? N : 1));
	Cells *c = syst.cells;
	for(int i = 0; i < N; i++) {
		PatchyParticle *p = syst.particles + i;
		int nb = 0, no = 0, ind[3], loop_ind[3];
		cells_fill_and_get_idx_from_particle(&syst, p, ind);
		for(int j = -1; j < 2; j++) {
			loop_ind[0] = (ind[0] + j + c->N_side[0]) % c->N_side[0];
			for(int k = -1; k < 2; k++) {
				loop_ind[1] = (ind[1] + k + c->N_side[1]) % c->N_side[1];
				for(int l = -1; l < 2; l++) {
					loop_ind[2] = (ind[2] + l + c->N_side[2]) % c->N_side[2];
					int loop_index = (loop_ind[0] * c->N_side[1] + loop_ind[1]) * c->N_side[2] + loop_ind[2];
					PatchyParticle *q = c->heads[loop_index];
					while(q != NULL) {
						if(q->index != p->index) {
							int pp, pq;
							int val = MC_interact(&syst, p, q, &pp, &pq);
							if(val == PATCH_BOND) bonded[nb++] = q->index;
							else if(val == OVERLAP) overl[no++] = q->index;
						}
						q = c->next[q->index];
					}
				}
			}
		}
		qsort(bonded, nb, sizeof(int), cmp_int);
		qsort(overl, no, sizeof(int), cmp_int);
		printf("%d %.17g %d %d %d :", i, E[i], ov[i], nb, no);
		for(int t = 0; t < nb; t++) printf(" %d", bonded[t]);
		printf(" |");
		for(int t = 0; t < no; t++) printf(" %d", overl[t]);
		printf("\n");
	}
	free(E);
	free(ov);
	free(bonded);
	free(overl);
	system_free(&syst);
	cleanInputFile(&input);
	return 0;
}
