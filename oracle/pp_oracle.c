/*
 * pp_oracle.c -- CPU restatement of the PatchyParticles roto-translation MC path. TEST INFRASTRUCTURE:
 * see pp_oracle.h for who may use it and how it is pinned. Each routine names the reference routine it
 * restates (file:line inside the reference project) and keeps its floating-point operation order; the
 * build uses -ffp-contract=off. Parity is pinned against the reference built from source (oracle/_ref)
 * and against tests/golden/ outputs of that build.
 */
#include "pp_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

struct orc_system {
	orc_params prm;
	int N;
	double box[3];
	double V;
	double energy;
	double kf_sqr_rcut;
	double r_cut;
	int overlap;
	long long tries[ORC_N_MOVES];
	long long accepted[ORC_N_MOVES];
	double *r, *r_old;  /* N x 3 */
	double *R, *R_old;  /* N x 9, row-major: R[i*9 + 3*row + col] */
	double *patch;      /* N x 12 */
	double base[4][3];
	/* linked-list cells (cells.h:16-21) */
	int nside[3];
	int ncells;
	int *head, *next, *cell, *cell_old;
	/* drand48 state X (48 bits) */
	unsigned long long X;
	/* GC / SUS: particle capacity, SUS histogram, the full-system stop */
	int cap;
	long long *sus_hist;
	int error;
	/* base_orient (defs.h:71-74, system.c:33-54) and the AVB state (avb.h: avbmc) */
	double base_orient[9];
	double avb_vin, avb_vout, avb_p;
	int avb_status;
	int avb_nb[4]; /* neighbours[patch of the receiver]: bonded particle, or -1 (avb.c:43-75) */
	int avb_nn;    /* num_neighbours */
	/* VMMC state (vmmc.h: vmmc_d) */
	int *vm_links;   /* possible_links: pairs (lower index, higher index), capacity 16 cap */
	int vm_nlinks;
	int *vm_counter; /* possible_links_counter */
	int *vm_copies;  /* copies */
	int *vm_in;      /* is_in_cluster */
	int *vm_clust, vm_nclust;
	int *vm_pre, vm_npre;   /* prelinked_particles */
	int *vm_fail, vm_nfail; /* outright_failed */
	int vm_rot;             /* which_move: 1 rotation, 0 translation */
	double vm_R[9];         /* the move's rotation */
	double vm_move[3];      /* the move's translation */
	int vm_error;
};

/* ---------------------------------------------------------------- drand48 (POSIX recurrence) */
/* X <- (0x5DEECE66D X + 0xB) mod 2^48, returned as X / 2^48; srand48(s) sets X = (s & 0xffffffff) << 16 | 0x330E. */
static void orc_seed(orc_system *s, int seed) {
	s->X = ((unsigned long long) (unsigned int) seed << 16) | 0x330EULL;
}

static double orc_drand(orc_system *s) {
	s->X = (0x5DEECE66DULL * s->X + 0xBULL) & 0xFFFFFFFFFFFFULL;
	return (double) s->X * 0x1p-48;
}

void orc_drand48_sequence(int seed, int n, double *out) {
	orc_system tmp;
	orc_seed(&tmp, seed);
	for(int i = 0; i < n; i++) out[i] = orc_drand(&tmp);
}

/* ---------------------------------------------------------------- vector helpers (utils.c, utils.h) */
#define O_SCALAR(x, y) ((x)[0] * (y)[0] + (x)[1] * (y)[1] + (x)[2] * (y)[2]) /* utils.h:15 */

static void o_normalize(double *v) { /* utils.c:31-36 */
	double norm = sqrt(O_SCALAR(v, v));
	v[0] /= norm;
	v[1] /= norm;
	v[2] /= norm;
}

static void o_cross(const double *a, const double *b, double *res) { /* utils.c:25-29 */
	res[0] = a[1] * b[2] - a[2] * b[1];
	res[1] = a[2] * b[0] - a[0] * b[2];
	res[2] = a[0] * b[1] - a[1] * b[0];
}

static void o_gram_schmidt(double *v1, double *v2, double *v3) { /* utils.c:91-113 */
	double v1_norm2 = O_SCALAR(v1, v1);
	double v2_v1 = O_SCALAR(v2, v1);
	double b1 = v2_v1 / v1_norm2;
	for(int k = 0; k < 3; k++) v2[k] -= b1 * v1[k];
	double v3_v1 = O_SCALAR(v3, v1);
	double v3_v2 = O_SCALAR(v3, v2);
	double v2_norm2 = O_SCALAR(v2, v2);
	b1 = v3_v1 / v1_norm2;
	double b2 = v3_v2 / v2_norm2;
	for(int k = 0; k < 3; k++) v3[k] -= b1 * v1[k] + b2 * v2[k];
	o_normalize(v1);
	o_normalize(v2);
	o_normalize(v3);
}

static void o_random_vector_on_sphere(orc_system *s, double *res);

/* determinant (utils.c:78-89), same term order */
static double o_determinant(const double *m) {
	double det = 0.;
	det += m[0] * m[4] * m[8];
	det += m[1] * m[5] * m[6];
	det += m[2] * m[3] * m[7];
	det -= m[2] * m[4] * m[6];
	det -= m[0] * m[5] * m[7];
	det -= m[1] * m[3] * m[8];
	return det;
}

/* random_orientation (utils.c:133-169): three vectors on the sphere, Gram-Schmidt, rows (v3, v1, v2),
 * rows 0 and 1 swapped back when the determinant is negative */
static void o_random_orientation(orc_system *s, double *R) {
	double v1[3], v2[3], v3[3];
	o_random_vector_on_sphere(s, v1);
	o_random_vector_on_sphere(s, v2);
	o_random_vector_on_sphere(s, v3);
	o_gram_schmidt(v1, v2, v3);
	memcpy(R, v3, sizeof(v3));
	memcpy(R + 3, v1, sizeof(v1));
	memcpy(R + 6, v2, sizeof(v2));
	if(o_determinant(R) < 0.) {
		memcpy(R, v1, sizeof(v1));
		memcpy(R + 3, v3, sizeof(v3));
	}
}

/* make_initial_conf (generator.c:43-68) with main's box (generator.c:99-105), random numbers from
 * srand48(seed): uniform insertion in a cubic box of side (N / density)^(1/3), rejected when it overlaps
 * (r^2 < 1) an inserted particle in the 27 cells of edge >= 1 around it (cells.c:17-49), orientation from
 * random_orientation. Returns 0, or -1 for density outside (0, 0.7] (generator.c:99-102) or no memory. */
int orc_generate(int N, double density, int seed, double *r, double *R, double box[3]) {
	if(N < 0 || !(density > 0.) || density > 0.7) return -1;
	const double L = pow(N / density, 1. / 3.);
	orc_system g;
	orc_seed(&g, seed);
	int ns = (int) floor(L / 1.);
	if(ns < 3) ns = 3;
	const long long nc = (long long) ns * ns * ns;
	int *head = malloc(sizeof(int) * nc), *next = malloc(sizeof(int) * (N > 0 ? N : 1));
	if(head == NULL || next == NULL) {
		free(head);
		free(next);
		return -1;
	}
	for(long long c = 0; c < nc; c++) head[c] = -1;
	const double b[3] = { L, L, L };
	int inserted = 0;
	while(inserted < N) {
		double p[3];
		p[0] = orc_drand(&g) * L;
		p[1] = orc_drand(&g) * L;
		p[2] = orc_drand(&g) * L;
		int ind[3];
		for(int k = 0; k < 3; k++) ind[k] = (int) ((p[k] / b[k] - floor(p[k] / b[k])) * (1. - DBL_EPSILON) * ns);
		int overlap = 0;
		for(int j = -1; j < 2 && !overlap; j++)
			for(int k = -1; k < 2 && !overlap; k++)
				for(int l = -1; l < 2 && !overlap; l++) {
					const int cx = (ind[0] + j + ns) % ns, cy = (ind[1] + k + ns) % ns, cz = (ind[2] + l + ns) % ns;
					for(int q = head[((long long) cx * ns + cy) * ns + cz]; q != -1; q = next[q]) {
						double d[3];
						for(int a = 0; a < 3; a++) {
							d[a] = r[3 * (size_t) q + a] - p[a];
							d[a] -= b[a] * rint(d[a] / b[a]);
						}
						if(O_SCALAR(d, d) < 1.) {
							overlap = 1;
							break;
						}
					}
				}
		if(overlap) continue;
		o_random_orientation(&g, R + 9 * (size_t) inserted);
		memcpy(r + 3 * (size_t) inserted, p, sizeof(p));
		const int c = (ind[0] * ns + ind[1]) * ns + ind[2];
		next[inserted] = head[c];
		head[c] = inserted;
		inserted++;
	}
	free(head);
	free(next);
	box[0] = box[1] = box[2] = L;
	return 0;
}

/* patches[i] = R . base[i] with the MATRIX_VECTOR_MULTIPLICATION order (utils.h:17-21) */
static void o_set_patches(orc_system *s, int p) {
	const double *R = s->R + 9 * p;
	double *P = s->patch + 12 * p;
	for(int i = 0; i < 4; i++) {
		const double *b = s->base[i];
		P[3 * i + 0] = R[0] * b[0] + R[1] * b[1] + R[2] * b[2];
		P[3 * i + 1] = R[3] * b[0] + R[4] * b[1] + R[5] * b[2];
		P[3 * i + 2] = R[6] * b[0] + R[7] * b[1] + R[8] * b[2];
	}
}

/* random_vector_on_sphere (utils.c:115-131): Marsaglia (1972) rejection on the unit disc */
static void o_random_vector_on_sphere(orc_system *s, double *res) {
	double ran1, ran2, ransq;
	do {
		ran1 = 1. - 2. * orc_drand(s);
		ran2 = 1. - 2. * orc_drand(s);
		ransq = ran1 * ran1 + ran2 * ran2;
	} while(ransq >= 1.);
	double ranh = 2. * sqrt(1. - ransq);
	res[0] = ran1 * ranh;
	res[1] = ran2 * ranh;
	res[2] = 1. - 2. * ransq;
}

/* get_rotation_matrix (utils.c:186-202): rotation by t about the unit axis a, rows */
static void o_rotation_matrix(const double *a, double t, double *m) {
	double st = sin(t);
	double ct = cos(t);
	double uct = 1. - ct;
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

/* matrix_matrix_multiplication (utils.c:172-184): out = m . n (out may not alias m or n) */
static void o_matmul(const double *m, const double *n, double *out) {
	for(int i = 0; i < 3; i++)
		for(int j = 0; j < 3; j++) out[3 * i + j] = m[3 * i + 0] * n[0 + j] + m[3 * i + 1] * n[3 + j] + m[3 * i + 2] * n[6 + j];
}

/* MATRIX_VECTOR_MULTIPLICATION (utils.h:17-21): res = m . v */
static void o_matvec(const double *m, const double *v, double *res) {
	res[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
	res[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
	res[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}

/* utils_rotate_matrix (utils.c:204-209): new = old . Rot(axis, t) */
static void o_rotate_matrix(const double *old, double *out, const double *a, double t) {
	double m[9];
	o_rotation_matrix(a, t, m);
	o_matmul(old, m, out);
}

/* rotate_vector (utils.c:217-223, get_rotated_vector utils.c:211-215): v = Rot(axis, t) . v */
static void o_rotate_vector(double *v, const double *axis, double t) {
	double m[9], tmp[3];
	o_rotation_matrix(axis, t, m);
	o_matvec(m, v, tmp);
	memcpy(v, tmp, sizeof(tmp));
}

/* get_perpendicular_versor (utils.c:38-50): a random unit vector perpendicular to v */
static void o_perpendicular_versor(orc_system *s, const double *v, double *res) {
	o_random_vector_on_sphere(s, res);
	double v_norm2 = O_SCALAR(v, v);
	double res_v = O_SCALAR(res, v);
	double buffer = res_v / v_norm2;
	res[0] -= buffer * v[0];
	res[1] -= buffer * v[1];
	res[2] -= buffer * v[2];
	o_normalize(res);
}

/* set_orientation_around_vector (utils.c:225-270): orient = B . orient, B's third column along -v turned by
 * t about a random axis perpendicular to it */
static void o_set_orientation_around_vector(orc_system *s, const double *v, double *orient, double t) {
	double y_tmp[3] = { -v[0], -v[1], -v[2] }, w_tmp[3], z[3];
	o_random_vector_on_sphere(s, z);
	o_random_vector_on_sphere(s, w_tmp);
	o_gram_schmidt(y_tmp, z, w_tmp);
	double m[9], y[3], w[3];
	o_rotation_matrix(z, t, m);
	o_matvec(m, y_tmp, y);
	o_matvec(m, w_tmp, w);
	double B[9] = { z[0], w[0], y[0], z[1], w[1], y[1], z[2], w[2], y[2] }; /* columns z, w, y */
	if(o_determinant(B) < 0) {
		B[0] = w[0];
		B[3] = w[1];
		B[6] = w[2];
		B[1] = z[0];
		B[4] = z[1];
		B[7] = z[2];
	}
	double old[9];
	memcpy(old, orient, sizeof(old));
	o_matmul(B, old, orient);
}

void orc_base_patches(double base[4][3]) { /* _init_tetrahedral_patches, system.c:20-31 */
	double h = 0.5 / sqrt(3.);
	double v[4][3] = { { -h, -h, h }, { h, -h, -h }, { h, h, h }, { -h, h, -h } };
	for(int i = 0; i < 4; i++) {
		o_normalize(v[i]);
		memcpy(base[i], v[i], sizeof(v[i]));
	}
}

/* ---------------------------------------------------------------- cells (cells.c) */
static int o_cell_index(const orc_system *s, const double *r, int idx[3]) { /* cells.c:43-49 */
	for(int k = 0; k < 3; k++) idx[k] = (int) ((r[k] / s->box[k] - floor(r[k] / s->box[k])) * (1. - DBL_EPSILON) * s->nside[k]);
	return (idx[0] * s->nside[1] + idx[1]) * s->nside[2] + idx[2];
}

static int o_cells_init(orc_system *s) { /* cells.c:17-37 */
	for(int k = 0; k < 3; k++) {
		s->nside[k] = floor(s->box[k] / s->r_cut);
		if(s->nside[k] < 3) s->nside[k] = 3;
	}
	s->ncells = s->nside[0] * s->nside[1] * s->nside[2];
	free(s->head);
	s->head = malloc(sizeof(int) * s->ncells);
	if(s->head == NULL) return -1;
	for(int i = 0; i < s->ncells; i++) s->head[i] = -1;
	for(int i = 0; i < s->N; i++) s->next[i] = -1;
	return 0;
}

static void o_cells_fill(orc_system *s) { /* cells.c:51-63 */
	int ind[3];
	for(int i = 0; i < s->N; i++) {
		int c = o_cell_index(s, s->r + 3 * i, ind);
		s->next[i] = s->head[c];
		s->head[c] = i;
		s->cell[i] = c;
		s->cell_old[i] = c;
	}
}

static void o_unlink(orc_system *s, int p, int c) {
	if(s->head[c] == p) s->head[c] = s->next[p];
	else {
		int q = s->head[c];
		while(s->next[q] != p) q = s->next[q];
		s->next[q] = s->next[p];
	}
}

static void o_change_cell(orc_system *s, int p) { /* MC_change_cell, MC.c:180-206 */
	int ind[3];
	int c = o_cell_index(s, s->r + 3 * p, ind);
	if(c == s->cell[p]) {
		s->cell_old[p] = s->cell[p];
		return;
	}
	o_unlink(s, p, s->cell[p]);
	s->next[p] = s->head[c];
	s->head[c] = p;
	s->cell_old[p] = s->cell[p];
	s->cell[p] = c;
}

/* ---------------------------------------------------------------- pair interaction and energy (MC.c) */
/* MC_would_interact (MC.c:232-266): q's position r and patches qp, seen from particle p */
static int o_would_interact(const orc_system *s, int p, const double *r, const double *qp) {
	const double *rp = s->r + 3 * p;
	double d[3] = { r[0] - rp[0], r[1] - rp[1], r[2] - rp[2] };
	d[0] -= s->box[0] * rint(d[0] / s->box[0]);
	d[1] -= s->box[1] * rint(d[1] / s->box[1]);
	d[2] -= s->box[2] * rint(d[2] / s->box[2]);
	double dist2 = O_SCALAR(d, d);
	if(dist2 < 1.) return ORC_OVERLAP;
	if(dist2 < s->kf_sqr_rcut) {
		double norm = sqrt(dist2);
		d[0] /= norm;
		d[1] /= norm;
		d[2] /= norm;
		const double *pp = s->patch + 12 * p;
		for(int a = 0; a < 4; a++) {
			double p_cos = O_SCALAR(d, pp + 3 * a);
			if(p_cos > s->prm.kf_cosmax) {
				for(int b = 0; b < 4; b++) {
					double q_cos = -O_SCALAR(d, qp + 3 * b);
					if(q_cos > s->prm.kf_cosmax) return ORC_PATCH_BOND;
				}
			}
		}
	}
	return ORC_NO_BOND;
}

int orc_interact(orc_system *s, int i, int j) { /* MC_interact, MC.c:268-270 */
	return o_would_interact(s, i, s->r + 3 * j, s->patch + 12 * j);
}

static double o_energy(orc_system *s, int p) { /* MC_energy, MC.c:272-309 */
	s->overlap = 0;
	double E = 0.;
	int ind[3];
	o_cell_index(s, s->r + 3 * p, ind);
	for(int j = -1; j < 2; j++) {
		int cx = (ind[0] + j + s->nside[0]) % s->nside[0];
		for(int k = -1; k < 2; k++) {
			int cy = (ind[1] + k + s->nside[1]) % s->nside[1];
			for(int l = -1; l < 2; l++) {
				int cz = (ind[2] + l + s->nside[2]) % s->nside[2];
				int q = s->head[(cx * s->nside[1] + cy) * s->nside[2] + cz];
				while(q != -1) {
					if(q != p) {
						int val = orc_interact(s, p, q);
						if(val == ORC_PATCH_BOND) E -= 1.;
						else if(val == ORC_OVERLAP) {
							s->overlap = 1;
							return 0.;
						}
					}
					q = s->next[q];
				}
			}
		}
	}
	return E;
}

double orc_particle_energy(orc_system *s, int i, int *overlap) {
	double E = o_energy(s, i);
	if(overlap) *overlap = s->overlap;
	return E;
}

/* full 27-cell walk of particle p without early exit (as output_print_bonds, output.c:213-268) */
static void o_partners(orc_system *s, int p, int *nb, int *no, int *bonded, int cap) {
	int ind[3];
	*nb = *no = 0;
	o_cell_index(s, s->r + 3 * p, ind);
	for(int j = -1; j < 2; j++) {
		int cx = (ind[0] + j + s->nside[0]) % s->nside[0];
		for(int k = -1; k < 2; k++) {
			int cy = (ind[1] + k + s->nside[1]) % s->nside[1];
			for(int l = -1; l < 2; l++) {
				int cz = (ind[2] + l + s->nside[2]) % s->nside[2];
				int q = s->head[(cx * s->nside[1] + cy) * s->nside[2] + cz];
				while(q != -1) {
					if(q != p) {
						int val = orc_interact(s, p, q);
						if(val == ORC_PATCH_BOND) {
							if(bonded != NULL && *nb < cap) bonded[*nb] = q;
							(*nb)++;
						}
						else if(val == ORC_OVERLAP) (*no)++;
					}
					q = s->next[q];
				}
			}
		}
	}
}

double orc_energies(orc_system *s, double *E, int *overlap, int *n_bonds, int *n_overlaps) {
	double tot = 0.;
	for(int i = 0; i < s->N; i++) {
		double e = o_energy(s, i);
		if(E) E[i] = e;
		if(overlap) overlap[i] = s->overlap;
		tot += e;
		if(n_bonds || n_overlaps) {
			int nb, no;
			o_partners(s, i, &nb, &no, NULL, 0);
			if(n_bonds) n_bonds[i] = nb;
			if(n_overlaps) n_overlaps[i] = no;
		}
	}
	return tot * 0.5;
}

static int cmp_int(const void *a, const void *b) {
	int x = *(const int *) a, y = *(const int *) b;
	return (x > y) - (x < y);
}

int orc_bond_lists(orc_system *s, int *offsets, int *partners, int cap) {
	int total = 0;
	for(int i = 0; i < s->N; i++) {
		int nb, no;
		offsets[i] = total;
		o_partners(s, i, &nb, &no, partners + total, cap - total);
		if(total + nb > cap) return -1;
		qsort(partners + total, nb, sizeof(int), cmp_int);
		total += nb;
	}
	offsets[s->N] = total;
	return total;
}

/* ---------------------------------------------------------------- moves (MC.c) */
static void o_rototranslate(orc_system *s, int p, const double *disp, const double *newR) { /* MC.c:208-230 */
	double *r = s->r + 3 * p, *ro = s->r_old + 3 * p;
	for(int k = 0; k < 3; k++) {
		ro[k] = r[k];
		r[k] += disp[k];
	}
	memcpy(s->R_old + 9 * p, s->R + 9 * p, 9 * sizeof(double));
	memcpy(s->R + 9 * p, newR, 9 * sizeof(double));
	o_set_patches(s, p);
	o_change_cell(s, p);
}

static void o_rollback(orc_system *s, int p) { /* MC_rollback_particle, MC.c:146-178 */
	memcpy(s->r + 3 * p, s->r_old + 3 * p, 3 * sizeof(double));
	memcpy(s->R + 9 * p, s->R_old + 9 * p, 9 * sizeof(double));
	o_set_patches(s, p);
	if(s->cell[p] != s->cell_old[p]) {
		o_unlink(s, p, s->cell[p]);
		s->next[p] = s->head[s->cell_old[p]];
		s->head[s->cell_old[p]] = p;
		int c = s->cell[p];
		s->cell[p] = s->cell_old[p];
		s->cell_old[p] = c;
	}
}

static void o_move_rototranslate(orc_system *s) { /* MC_move_rototranslate, MC.c:311-340 */
	int p = (int) (orc_drand(s) * s->N);
	s->tries[ORC_ROTO_TRASL]++;
	double disp[3];
	disp[0] = (orc_drand(s) - 0.5) * s->prm.disp_max;
	disp[1] = (orc_drand(s) - 0.5) * s->prm.disp_max;
	disp[2] = (orc_drand(s) - 0.5) * s->prm.disp_max;
	double theta = orc_drand(s) * s->prm.theta_max;
	double axis[3], newR[9];
	o_random_vector_on_sphere(s, axis);
	o_rotate_matrix(s->R + 9 * p, newR, axis, theta);

	double dE = -o_energy(s, p);
	o_rototranslate(s, p, disp, newR);
	dE += o_energy(s, p);

	if(!s->overlap && (dE < 0. || orc_drand(s) < exp(-dE / s->prm.T))) {
		s->energy += dE;
		s->accepted[ORC_ROTO_TRASL]++;
	}
	else {
		o_rollback(s, p);
		s->overlap = 0;
	}
}

/* MC_would_interact (MC.c:232-266) with the bonding patches: *pp / *qp receive the first (p patch, q patch)
 * pair, p's patches outer, that bonds */
static int o_would_interact_patches(const orc_system *s, int p, const double *r, const double *qpatch, int *pp, int *qp) {
	const double *rp = s->r + 3 * p;
	double d[3] = { r[0] - rp[0], r[1] - rp[1], r[2] - rp[2] };
	d[0] -= s->box[0] * rint(d[0] / s->box[0]);
	d[1] -= s->box[1] * rint(d[1] / s->box[1]);
	d[2] -= s->box[2] * rint(d[2] / s->box[2]);
	double dist2 = O_SCALAR(d, d);
	if(dist2 < 1.) return ORC_OVERLAP;
	if(dist2 < s->kf_sqr_rcut) {
		double norm = sqrt(dist2);
		d[0] /= norm;
		d[1] /= norm;
		d[2] /= norm;
		const double *pa = s->patch + 12 * p;
		for(int a = 0; a < 4; a++) {
			double p_cos = O_SCALAR(d, pa + 3 * a);
			if(p_cos > s->prm.kf_cosmax) {
				for(int b = 0; b < 4; b++) {
					double q_cos = -O_SCALAR(d, qpatch + 3 * b);
					if(q_cos > s->prm.kf_cosmax) {
						*pp = a;
						*qp = b;
						return ORC_PATCH_BOND;
					}
				}
			}
		}
	}
	return ORC_NO_BOND;
}

/* _set_neighbours (avb.c:43-75): the particles bonded to p, indexed by p's bonding patch */
static void o_avb_set_neighbours(orc_system *s, int p) {
	int ind[3];
	o_cell_index(s, s->r + 3 * p, ind);
	s->avb_nn = 0;
	for(int k = 0; k < 4; k++) s->avb_nb[k] = -1;
	for(int j = -1; j < 2; j++) {
		int cx = (ind[0] + j + s->nside[0]) % s->nside[0];
		for(int k = -1; k < 2; k++) {
			int cy = (ind[1] + k + s->nside[1]) % s->nside[1];
			for(int l = -1; l < 2; l++) {
				int cz = (ind[2] + l + s->nside[2]) % s->nside[2];
				int q = s->head[(cx * s->nside[1] + cy) * s->nside[2] + cz];
				while(q != -1) {
					if(q != p) {
						int pp = 0, qp = 0;
						if(o_would_interact_patches(s, p, s->r + 3 * q, s->patch + 12 * q, &pp, &qp) == ORC_PATCH_BOND) {
							s->avb_nb[pp] = q;
							s->avb_nn++;
						}
					}
					q = s->next[q];
				}
			}
		}
	}
}

/* place_inside_vbonding (utils.c:52-76): a position and orientation inside the bonding volume of patch
 * target_patch of particle rec */
static void o_place_inside_vbonding(orc_system *s, int rec, double *r, double *orient, int target_patch) {
	o_rotate_matrix(s->base_orient, orient, s->base[0], 2 * orc_drand(s) * M_PI);
	double dir[3];
	memcpy(dir, s->patch + 12 * rec + 3 * target_patch, sizeof(dir));
	double norm_vect[3];
	o_perpendicular_versor(s, dir, norm_vect);
	double theta = acos(s->prm.kf_cosmax + (1. - s->prm.kf_cosmax) * orc_drand(s));
	o_rotate_vector(dir, norm_vect, theta);
	o_normalize(dir);
	double theta2 = acos(s->prm.kf_cosmax + (1. - s->prm.kf_cosmax) * orc_drand(s));
	o_set_orientation_around_vector(s, dir, orient, theta2);
	const double dl = s->prm.kf_delta;
	double dist = pow(1. + orc_drand(s) * (dl * dl * dl + 3. * (dl * dl) + 3. * dl), 1. / 3.);
	const double *rr = s->r + 3 * rec;
	r[0] = dir[0] * dist + rr[0];
	r[1] = dir[1] * dist + rr[1];
	r[2] = dir[2] * dist + rr[2];
}

/* AVBMC_dynamics (avb.c:77-186): with probability avb_p (or for N < 2) a roto-translation, otherwise an
 * aggregation-volume-bias move of a particle into or out of the bonding volume of a random receiver */
static void o_avb_dynamics(orc_system *s) {
	if(orc_drand(s) < s->avb_p || s->N < 2) {
		o_move_rototranslate(s);
		return;
	}
	s->tries[ORC_AVB]++;
	const int rec = (int) (orc_drand(s) * s->N);
	o_avb_set_neighbours(s, rec);
	int p;
	if(orc_drand(s) > 0.5) { /* into the bonding volume */
		if(s->avb_nn == s->N - 1) return;
		int found;
		do {
			p = (int) (orc_drand(s) * s->N);
			found = 1;
			for(int i = 0; i < 4 && found; i++)
				if(s->avb_nb[i] == p) found = 0;
		} while(!found || p == rec);
		double new_r[3], new_R[9];
		int target_patch = (int) (orc_drand(s) * 4);
		o_place_inside_vbonding(s, rec, new_r, new_R, target_patch);
		const double *rp = s->r + 3 * p;
		double disp[3] = { new_r[0] - rp[0], new_r[1] - rp[1], new_r[2] - rp[2] };
		double dE = -o_energy(s, p);
		o_rototranslate(s, p, disp, new_R);
		dE += o_energy(s, p);
		double acc = exp(-dE / s->prm.T) * (s->N - s->avb_nn - 1.) * s->avb_vin / ((s->avb_nn + 1.) * s->avb_vout);
		if(!s->overlap && orc_drand(s) < acc) {
			s->accepted[ORC_AVB]++;
			s->energy += dE;
		}
		else o_rollback(s, p); /* the reference leaves syst->overlap set here; every MC_energy clears it */
	}
	else { /* out of the bonding volume */
		if(s->avb_nn == 0) return;
		int random_neighbour = (int) (orc_drand(s) * s->avb_nn);
		int cn = 0, ci = 0;
		while(cn <= random_neighbour) {
			if(s->avb_nb[ci] != -1) cn++;
			ci++;
		}
		p = s->avb_nb[ci - 1];
		double new_r[3], new_R[9], new_patches[12];
		int buff;
		do {
			new_r[0] = orc_drand(s) * s->box[0];
			new_r[1] = orc_drand(s) * s->box[1];
			new_r[2] = orc_drand(s) * s->box[2];
			o_random_orientation(s, new_R);
			for(int i = 0; i < 4; i++) o_matvec(new_R, s->base[i], new_patches + 3 * i);
		} while(o_would_interact_patches(s, rec, new_r, new_patches, &buff, &buff) == ORC_PATCH_BOND);
		const double *rp = s->r + 3 * p;
		double disp[3] = { new_r[0] - rp[0], new_r[1] - rp[1], new_r[2] - rp[2] };
		double dE = -o_energy(s, p);
		o_rototranslate(s, p, disp, new_R);
		dE += o_energy(s, p);
		double acc = exp(-dE / s->prm.T) * s->avb_nn * s->avb_vout / ((s->N - s->avb_nn) * s->avb_vin);
		if(!s->overlap && orc_drand(s) < acc) {
			s->accepted[ORC_AVB]++;
			s->energy += dE;
		}
		else o_rollback(s, p);
	}
}

/* ---------------------------------------------------------------- VMMC (vmmc.c) */
/* _store_dof / _restore_dof (vmmc.c:58-79) */
static void o_store_dof(orc_system *s, int p) {
	memcpy(s->r_old + 3 * p, s->r + 3 * p, 3 * sizeof(double));
	memcpy(s->R_old + 9 * p, s->R + 9 * p, 9 * sizeof(double));
}

static void o_restore_dof(orc_system *s, int p) {
	memcpy(s->r + 3 * p, s->r_old + 3 * p, 3 * sizeof(double));
	memcpy(s->R + 9 * p, s->R_old + 9 * p, 9 * sizeof(double));
	o_set_patches(s, p);
}

/* _pair_energy (vmmc.c:81-95) */
static double o_pair_energy(orc_system *s, int p, int q) {
	int val = orc_interact(s, p, q);
	if(val == ORC_PATCH_BOND) return -1.;
	if(val == ORC_OVERLAP) s->overlap = 1;
	return 0.;
}

/* _compute_cluster_energy (vmmc.c:107-137): the cluster's bonds to particles outside it */
static double o_cluster_energy(orc_system *s) {
	double res = 0.;
	for(int i = 0; i < s->vm_nclust; i++) {
		int p = s->vm_clust[i];
		int ind[3];
		o_cell_index(s, s->r + 3 * p, ind);
		for(int j = -1; j < 2; j++) {
			int cx = (ind[0] + j + s->nside[0]) % s->nside[0];
			for(int k = -1; k < 2; k++) {
				int cy = (ind[1] + k + s->nside[1]) % s->nside[1];
				for(int l = -1; l < 2; l++) {
					int cz = (ind[2] + l + s->nside[2]) % s->nside[2];
					int q = s->head[(cx * s->nside[1] + cy) * s->nside[2] + cz];
					while(q != -1) {
						if(s->vm_in[q] == 0) res += o_pair_energy(s, p, q);
						q = s->next[q];
					}
				}
			}
		}
	}
	return res;
}

/* _move_particle (vmmc.c:231-256): the translation, or the rotation about the seed */
static void o_vmmc_move(orc_system *s, int p) {
	double *r = s->r + 3 * p;
	if(!s->vm_rot) {
		r[0] += s->vm_move[0];
		r[1] += s->vm_move[1];
		r[2] += s->vm_move[2];
		return;
	}
	const double *seed = s->r + 3 * s->vm_clust[0];
	double dr_tmp[3] = { r[0] - seed[0], r[1] - seed[1], r[2] - seed[2] }, dr[3];
	o_matvec(s->vm_R, dr_tmp, dr);
	r[0] = seed[0] + dr[0];
	r[1] = seed[1] + dr[1];
	r[2] = seed[2] + dr[2];
	o_matmul(s->vm_R, s->R_old + 9 * p, s->R + 9 * p);
	o_set_patches(s, p);
}

/* _populate_possible_links (vmmc.c:148-229): the links p can form at its current (real or virtual)
 * position, each partner taken at its image closest to p's real position */
static void o_populate_links(orc_system *s, int p, int *force_reject) {
	int ind[3];
	o_cell_index(s, s->r + 3 * p, ind);
	const double *rp = s->r + 3 * p, *rpo = s->r_old + 3 * p;
	for(int j = -1; j < 2; j++) {
		int cx = (ind[0] + j + s->nside[0]) % s->nside[0];
		for(int k = -1; k < 2; k++) {
			int cy = (ind[1] + k + s->nside[1]) % s->nside[1];
			for(int l = -1; l < 2; l++) {
				int cz = (ind[2] + l + s->nside[2]) % s->nside[2];
				int q = s->head[(cx * s->nside[1] + cy) * s->nside[2] + cz];
				while(q != -1) {
					if(q != p) {
						double *rq = s->r + 3 * q;
						double dist[3] = { rq[0] - rp[0], rq[1] - rp[1], rq[2] - rp[2] };
						dist[0] -= s->box[0] * rint(dist[0] / s->box[0]);
						dist[1] -= s->box[1] * rint(dist[1] / s->box[1]);
						dist[2] -= s->box[2] * rint(dist[2] / s->box[2]);
						double dist2 = O_SCALAR(dist, dist);
						if(dist2 < s->kf_sqr_rcut) {
							if(s->vm_nlinks >= 16 * s->cap) { /* output_exit "VMMC: memory exhausted" */
								s->vm_error = 1;
								*force_reject = 1;
								return;
							}
							/* normalized_diff_vector (vmmc.c:139-146) from p's real position */
							dist[0] = rq[0] - rpo[0];
							dist[1] = rq[1] - rpo[1];
							dist[2] = rq[2] - rpo[2];
							dist[0] -= s->box[0] * rint(dist[0] / s->box[0]);
							dist[1] -= s->box[1] * rint(dist[1] / s->box[1]);
							dist[2] -= s->box[2] * rint(dist[2] / s->box[2]);
							double new_pos[3] = { rpo[0] + dist[0], rpo[1] + dist[1], rpo[2] + dist[2] };
							if(s->vm_copies[q] == 1 || s->vm_in[q] == 1) {
								if(fabs(new_pos[0] - rq[0]) > 1e-6 || fabs(new_pos[1] - rq[1]) > 1e-6 || fabs(new_pos[2] - rq[2]) > 1e-6) {
									*force_reject = 1;
									return;
								}
							}
							if(s->vm_copies[q] == 0 && s->vm_in[q] == 0) {
								rq[0] = new_pos[0];
								rq[1] = new_pos[1];
								rq[2] = new_pos[2];
								s->vm_copies[q] = 1;
							}
							int n = s->vm_nlinks;
							s->vm_links[2 * n] = p < q ? p : q;
							s->vm_links[2 * n + 1] = p < q ? q : p;
							s->vm_nlinks++;
							s->vm_counter[p]++;
							s->vm_counter[q]++;
							/* a link already listed is dropped again (_mycomp, vmmc.c:97-105) */
							for(int m = 0; m < s->vm_nlinks - 1; m++) {
								if(s->vm_links[2 * m] == s->vm_links[2 * n] && s->vm_links[2 * m + 1] == s->vm_links[2 * n + 1]) {
									s->vm_nlinks--;
									s->vm_counter[p]--;
									s->vm_counter[q]--;
									if(s->vm_counter[p] == 0) s->vm_copies[p] = 0;
									if(s->vm_counter[q] == 0) s->vm_copies[q] = 0;
									break;
								}
							}
						}
					}
					q = s->next[q];
				}
			}
		}
	}
}

/* drops link k (the last one takes its place) and releases its particles' copies (vmmc.c:310-318, 386-397) */
static void o_drop_link(orc_system *s, int k, int p, int q) {
	s->vm_links[2 * k] = s->vm_links[2 * (s->vm_nlinks - 1)];
	s->vm_links[2 * k + 1] = s->vm_links[2 * (s->vm_nlinks - 1) + 1];
	s->vm_nlinks--;
	s->vm_counter[p]--;
	s->vm_counter[q]--;
	if(s->vm_counter[p] == 0) s->vm_copies[p] = 0;
	if(s->vm_counter[q] == 0) s->vm_copies[q] = 0;
}

/* VMMC_dynamics (vmmc.c:258-483) */
static void o_vmmc_dynamics(orc_system *s) {
	s->tries[ORC_MOVE_VMMC]++;
	int force_reject = 0;
	s->vm_nclust = 1;
	s->vm_nfail = 0;
	s->vm_nlinks = 0;
	s->vm_npre = 0;
	int seed = (int) (orc_drand(s) * s->N);
	s->vm_in[seed] = 1;
	s->vm_clust[0] = seed;
	if(orc_drand(s) < 0.5) {
		s->vm_rot = 0;
		s->vm_move[0] = (orc_drand(s) - 0.5) * s->prm.disp_max;
		s->vm_move[1] = (orc_drand(s) - 0.5) * s->prm.disp_max;
		s->vm_move[2] = (orc_drand(s) - 0.5) * s->prm.disp_max;
	}
	else {
		s->vm_rot = 1;
		o_random_vector_on_sphere(s, s->vm_move);
		double angle = orc_drand(s) * s->prm.theta_max;
		o_rotation_matrix(s->vm_move, angle, s->vm_R);
	}
	o_store_dof(s, seed);
	o_populate_links(s, seed, &force_reject);
	if(!force_reject) {
		o_vmmc_move(s, seed);
		o_populate_links(s, seed, &force_reject);
		o_restore_dof(s, seed);
	}
	while(s->vm_nlinks > 0 && s->vm_nclust < s->prm.vmmc_max_cluster && !force_reject) {
		int k = (int) (orc_drand(s) * s->vm_nlinks);
		int p = s->vm_links[2 * k], q = s->vm_links[2 * k + 1];
		if(s->vm_in[p] == 1 && s->vm_in[q] == 1) {
			o_drop_link(s, k, p, q);
			continue;
		}
		if(s->vm_in[p] == 0) {
			int t = q;
			q = p;
			p = t;
		}
		double E_old = o_pair_energy(s, p, q);
		o_store_dof(s, p);
		o_vmmc_move(s, p);
		double E_p_moved = o_pair_energy(s, p, q);
		o_restore_dof(s, p);
		int force_prelink = s->overlap;
		s->overlap = 0;
		double p1 = 1. - exp((1. / s->prm.T) * (E_old - E_p_moved));
		if(force_prelink == 1 || p1 > orc_drand(s)) {
			o_store_dof(s, q);
			o_vmmc_move(s, q);
			double E_q_moved = o_pair_energy(s, p, q);
			o_restore_dof(s, q);
			int force_link = s->overlap;
			s->overlap = 0;
			double p2 = 1. - exp((1. / s->prm.T) * (E_old - E_q_moved));
			if(p2 > 1.) p2 = 1.;
			if(force_link == 1 || (p2 / p1) > orc_drand(s)) {
				s->vm_copies[q] = 0;
				s->vm_in[q] = 1;
				s->vm_clust[s->vm_nclust++] = q;
				o_store_dof(s, q);
				o_populate_links(s, q, &force_reject);
				if(force_reject) break;
				o_vmmc_move(s, q);
				o_populate_links(s, q, &force_reject);
				o_restore_dof(s, q);
				if(force_reject) break;
			}
			else s->vm_pre[s->vm_npre++] = q;
		}
		else s->vm_fail[s->vm_nfail++] = q;
		o_drop_link(s, k, p, q);
	}
	if(s->vm_nclust == s->prm.vmmc_max_cluster) force_reject = 1;
	for(int i = 0; i < s->vm_npre; i++) {
		int p = s->vm_pre[i];
		if(s->vm_in[p] == 0) force_reject = 1;
		else s->vm_copies[p] = 0;
	}
	double deltaE = 0.;
	if(force_reject == 0) deltaE = -o_cluster_energy(s);
	if(s->overlap) s->vm_error = 1; /* assert(syst->overlap == 0), vmmc.c:436 */
	for(int i = 0; i < s->vm_nclust && !force_reject; i++) {
		int p = s->vm_clust[i];
		o_store_dof(s, p);
		o_vmmc_move(s, p);
		o_change_cell(s, p);
	}
	if(force_reject == 0) deltaE += o_cluster_energy(s);
	if(s->overlap) s->vm_error = 1; /* vmmc.c:446 */
	if(force_reject == 1)
		for(int i = 0; i < s->vm_nclust; i++) o_restore_dof(s, s->vm_clust[i]);
	if(force_reject == 0) {
		s->accepted[ORC_MOVE_VMMC]++;
		s->energy += deltaE;
	}
	for(int i = 0; i < s->vm_nclust; i++) {
		int p = s->vm_clust[i];
		o_change_cell(s, p);
		s->vm_in[p] = 0;
	}
	for(int i = 0; i < s->vm_nfail; i++) s->vm_copies[s->vm_fail[i]] = 0;
	s->vm_nfail = 0;
	for(int i = 0; i < s->vm_nlinks; i++) {
		int p = s->vm_links[2 * i], q = s->vm_links[2 * i + 1];
		s->vm_copies[p] = s->vm_copies[q] = 0;
		s->vm_counter[p] = s->vm_counter[q] = 0;
	}
}

int orc_vmmc_error(const orc_system *s) { return s->vm_error; }

/* syst->do_dynamics (MC_init, MC.c:115-130) */
static void o_dynamics(orc_system *s) {
	if(s->prm.dynamics == ORC_AVBMC) o_avb_dynamics(s);
	else if(s->prm.dynamics == ORC_VMMC) o_vmmc_dynamics(s);
	else o_move_rototranslate(s);
}

int orc_avb_status(const orc_system *s) { return s->avb_status; }

void orc_avb_volumes(const orc_system *s, double *v_in, double *v_out) {
	*v_in = s->avb_vin;
	*v_out = s->avb_vout;
}

static void o_change_volume(orc_system *s) { /* MC_change_volume, MC.c:450-513 */
	s->tries[ORC_VOLUME]++;
	double dE = -s->energy;
	double V0 = s->box[0] * s->box[1] * s->box[2];
	int dir = orc_drand(s) * 3;
	double lnV = log(V0) + (orc_drand(s) - 0.5) * s->prm.rescale_factor_max;
	double V1 = exp(lnV);
	double old_side = s->box[dir];
	double new_side = V1;
	for(int i = 0; i < 3; i++)
		if(i != dir) new_side /= s->box[i];
	s->box[dir] = new_side;
	double f = new_side / old_side;
	for(int i = 0; i < s->N; i++) s->r[3 * i + dir] *= f;

	if((s->box[dir] / s->nside[dir]) < s->r_cut) {
		o_cells_init(s);
		o_cells_fill(s);
	}

	int overlap_found = 0;
	for(int i = 0; i < s->N && !overlap_found; i++) {
		dE += o_energy(s, i) * 0.5;
		if(s->overlap) overlap_found = 1;
	}

	double dV = V1 - V0;
	double arg = -(s->prm.P * dV + dE) / s->prm.T + (s->N + 1) * log(f);
	if(!overlap_found && orc_drand(s) < exp(arg)) {
		s->V = V1;
		s->energy += dE;
		s->accepted[ORC_VOLUME]++;
	}
	else {
		for(int i = 0; i < s->N; i++) s->r[3 * i + dir] /= f;
		s->box[dir] = old_side;
		s->overlap = 0;
	}
}

/* MC_change_Lx (MC.c:515-585): Lx changes by a uniform amount, Ly = Lz follow at constant volume, every
 * coordinate is rescaled; accepted with probability min(1, exp(+dE / T)) (MC.c:562) as the reference does;
 * a rejected move divides the positions back */
static void o_change_lx(orc_system *s) {
	s->tries[ORC_LX]++;
	double dE = -s->energy;
	double old_sides[3] = { s->box[0], s->box[1], s->box[2] };
	s->box[0] += (orc_drand(s) - 0.5) * s->prm.lx_change_max;
	s->box[1] = s->box[2] = sqrt(s->V / s->box[0]);
	if(s->box[1] < s->prm.lyz_min || s->box[1] > s->prm.lyz_max) { /* early rejection (MC.c:526-530) */
		memcpy(s->box, old_sides, sizeof(old_sides));
		return;
	}
	double f[3] = { s->box[0] / old_sides[0], s->box[1] / old_sides[1], s->box[2] / old_sides[2] };
	for(int i = 0; i < s->N; i++)
		for(int k = 0; k < 3; k++) s->r[3 * i + k] *= f[k];
	if((s->box[0] / s->nside[0]) < s->r_cut || (s->box[1] / s->nside[1]) < s->r_cut) {
		o_cells_init(s);
		o_cells_fill(s);
	}
	int overlap_found = 0;
	for(int i = 0; i < s->N && !overlap_found; i++) {
		dE += o_energy(s, i) * 0.5;
		if(s->overlap) overlap_found = 1;
	}
	if(!overlap_found && orc_drand(s) < exp(dE / s->prm.T)) {
		s->energy += dE;
		s->accepted[ORC_LX]++;
	}
	else {
		for(int i = 0; i < s->N; i++)
			for(int k = 0; k < 3; k++) s->r[3 * i + k] /= f[k];
		memcpy(s->box, old_sides, sizeof(old_sides));
		if((s->box[0] / s->nside[0]) < s->r_cut || (s->box[1] / s->nside[1]) < s->r_cut) {
			o_cells_init(s);
			o_cells_fill(s);
		}
		s->overlap = 0;
	}
}

/* MC_add_remove (MC.c:342-448): an insertion at a uniform position with a random orientation, accepted
 * with exp(-dE / T) z V / (N + 1), or the removal of a uniformly chosen particle, accepted with
 * exp(-dE / T) N / (V z); the last particle takes the removed one's index (and memory position) */
static void o_add_remove(orc_system *s) {
	if(orc_drand(s) < 0.5) {
		if(s->N == s->prm.n_max) {
			if(s->prm.ensemble == ORC_GC) s->error = 1; /* output_exit in the reference */
			return;
		}
		s->tries[ORC_ADD]++;
		const int p = s->N;
		double *r = s->r + 3 * p;
		r[0] = orc_drand(s) * s->box[0];
		r[1] = orc_drand(s) * s->box[1];
		r[2] = orc_drand(s) * s->box[2];
		o_random_orientation(s, s->R + 9 * p);
		o_set_patches(s, p);
		const double dE = o_energy(s, p);
		const double acc = exp(-dE / s->prm.T) * s->prm.activity * s->V / (s->N + 1.);
		if(!s->overlap && orc_drand(s) < acc) {
			s->energy += dE;
			int ind[3];
			const int c = o_cell_index(s, r, ind);
			s->next[p] = s->head[c];
			s->head[c] = p;
			s->cell[p] = s->cell_old[p] = c;
			s->N++;
			s->accepted[ORC_ADD]++;
		}
		else s->overlap = 0;
	}
	else {
		if(s->N == s->prm.n_min) return;
		s->tries[ORC_REMOVE]++;
		const int p = (int) (orc_drand(s) * s->N);
		const double dE = -o_energy(s, p);
		const double acc = exp(-dE / s->prm.T) * s->N / (s->V * s->prm.activity);
		if(orc_drand(s) < acc) {
			s->energy += dE;
			s->N--;
			o_unlink(s, p, s->cell[p]);
			if(p != s->N) {
				const int q = s->N;
				o_unlink(s, q, s->cell[q]);
				memcpy(s->r + 3 * p, s->r + 3 * q, 3 * sizeof(double));
				memcpy(s->R + 9 * p, s->R + 9 * q, 9 * sizeof(double));
				o_set_patches(s, p);
				s->cell[p] = s->cell[q];
				s->next[p] = s->head[s->cell[p]];
				s->head[s->cell[p]] = p;
			}
			s->accepted[ORC_REMOVE]++;
		}
	}
}

/* one iteration of the do_GC (MC.c:31-43) / do_SUS (MC.c:45-58) loop body */
static void o_attempt_gc(orc_system *s) {
	const double R = orc_drand(s);
	if(R < 0.01) {
		o_add_remove(s);
		if(s->prm.ensemble == ORC_SUS) s->sus_hist[s->N - s->prm.n_min]++;
	}
	else if(s->prm.lx_move && R < (0.01 + 1. / s->N)) o_change_lx(s);
	else if(s->N > 0) o_dynamics(s);
}

/* one iteration of the do_NVT (MC.c:19-29) or do_NPT (MC.c:60-68) loop body */
static void o_attempt(orc_system *s) {
	if(s->prm.ensemble == ORC_NPT) {
		if(orc_drand(s) < 1. / s->N) o_change_volume(s);
		else if(s->N > 0) o_dynamics(s);
	}
	else {
		o_dynamics(s);
		/* do_NVT always draws the Lx-move number (MC.c:24), even with Lx_move = 0 */
		const double R = orc_drand(s);
		if(s->prm.lx_move && R < 1. / s->N) o_change_lx(s);
	}
}

void orc_sweep(orc_system *s) {
	if(s->prm.dynamics == ORC_AVBMC && s->avb_status != 0) return; /* AVBMC_init refused the geometry */
	if(s->vm_error) return;
	if(s->prm.ensemble == ORC_GC || s->prm.ensemble == ORC_SUS) {
		for(int i = 0; i < s->prm.n_max && !s->error; i++) o_attempt_gc(s);
		return;
	}
	for(int i = 0; i < s->N && !s->vm_error; i++) o_attempt(s);
}

int orc_error(const orc_system *s) { return s->error; }

int orc_sus_hist(orc_system *s, long long *out, int reset) {
	const int n = s->prm.n_max - s->prm.n_min + 1;
	if(s->sus_hist == NULL) return 0;
	for(int i = 0; i < n; i++) {
		if(out) out[i] = s->sus_hist[i];
		if(reset) s->sus_hist[i] = 0;
	}
	return n;
}

void orc_sweeps(orc_system *s, long long n) {
	for(long long k = 0; k < n; k++) orc_sweep(s);
}

int orc_check_energy(orc_system *s) { /* MC_check_energy, MC.c:766-784 */
	double E = 0.;
	s->overlap = 0;
	for(int i = 0; i < s->N; i++) {
		E += o_energy(s, i);
		double *R = s->R + 9 * i;
		o_gram_schmidt(R, R + 3, R + 6);
	}
	E *= 0.5;
	/* as in the reference, only the last particle's overlap flag survives the loop */
	if(s->overlap) return -1;
	if(fabs(s->energy) > 1e-5 && fabs((E - s->energy) / s->energy) > 1e-5) return -2;
	s->energy = E;
	return 0;
}

/* ---------------------------------------------------------------- construction / IO */
static orc_system *o_alloc(int N, const orc_params *prm) {
	orc_system *s = calloc(1, sizeof(orc_system));
	if(s == NULL) return NULL;
	s->prm = *prm;
	s->N = N;
	/* GC / SUS systems keep room for n_max particles (system.c:199) */
	const int gc = prm->ensemble == ORC_GC || prm->ensemble == ORC_SUS;
	s->cap = gc && prm->n_max > N ? prm->n_max : N;
	if(prm->ensemble == ORC_GC) s->prm.n_min = 0;
	size_t n = s->cap > 0 ? (size_t) s->cap : 1;
	if(prm->ensemble == ORC_SUS) {
		s->sus_hist = calloc((size_t) (prm->n_max - prm->n_min + 1 > 0 ? prm->n_max - prm->n_min + 1 : 1), sizeof(long long));
		if(s->sus_hist == NULL) {
			free(s);
			return NULL;
		}
	}
	s->r = calloc(3 * n, sizeof(double));
	s->r_old = calloc(3 * n, sizeof(double));
	s->R = calloc(9 * n, sizeof(double));
	s->R_old = calloc(9 * n, sizeof(double));
	s->patch = calloc(12 * n, sizeof(double));
	s->next = malloc(n * sizeof(int));
	s->cell = malloc(n * sizeof(int));
	s->cell_old = malloc(n * sizeof(int));
	if(prm->dynamics == ORC_VMMC) { /* VMMC_init (vmmc.c:15-45) */
		s->vm_links = malloc(2 * 16 * n * sizeof(int));
		s->vm_counter = calloc(n, sizeof(int));
		s->vm_copies = calloc(n, sizeof(int));
		s->vm_in = calloc(n, sizeof(int));
		s->vm_clust = malloc(n * sizeof(int));
		s->vm_pre = malloc(n * sizeof(int));
		s->vm_fail = malloc(n * sizeof(int));
		if(!s->vm_links || !s->vm_counter || !s->vm_copies || !s->vm_in || !s->vm_clust || !s->vm_pre || !s->vm_fail) {
			orc_free(s);
			return NULL;
		}
	}
	if(!s->r || !s->r_old || !s->R || !s->R_old || !s->patch || !s->next || !s->cell || !s->cell_old) {
		orc_free(s);
		return NULL;
	}
	orc_base_patches(s->base);
	s->kf_sqr_rcut = (1. + prm->kf_delta) * (1. + prm->kf_delta); /* system.c:86 */
	s->r_cut = 1. + prm->kf_delta;                                /* system.c:249 */
	orc_seed(s, prm->seed);
	/* system_init seeds (system.c:75) and then _init_tetrahedral_patches builds base_orient
	 * (system.c:33-54): set_orientation_around_vector(-base_patches[0], identity, 0), transposed. Its two
	 * random unit vectors (utils.c:232-233) move the stream; the AVB move starts from base_orient. */
	double my[9] = { 1., 0., 0., 0., 1., 0., 0., 0., 1. };
	const double first[3] = { -s->base[0][0], -s->base[0][1], -s->base[0][2] };
	o_set_orientation_around_vector(s, first, my, 0.);
	for(int i = 0; i < 3; i++)
		for(int j = 0; j < 3; j++) s->base_orient[3 * i + j] = my[3 * j + i];
	return s;
}

static int o_finish(orc_system *s) {
	s->V = s->box[0] * s->box[1] * s->box[2];
	for(int i = 0; i < s->N; i++) o_set_patches(s, i);
	if(o_cells_init(s) != 0) return -1;
	o_cells_fill(s);
	s->energy = 0.;
	if(s->prm.dynamics == ORC_AVBMC) { /* AVBMC_init (avb.c:13-36), called from MC_init after system_init */
		const double dl = s->prm.kf_delta, cm = s->prm.kf_cosmax;
		double sin_theta = sin(acos(cm));
		s->avb_status = sin_theta >= 1. / (2. * (1. + dl)) ? -1 : 0;
		s->avb_vin = 4 * 4 * (M_PI * (dl * dl * dl + 3. * (dl * dl) + 3. * dl) * ((1. - cm) * (1. - cm)) / 3.);
		s->avb_vout = s->V - s->avb_vin;
		s->avb_p = s->prm.avb_p > 0. ? s->prm.avb_p : 0.5;
	}
	return 0;
}

orc_system *orc_load_rrr(const char *path, const orc_params *prm, char *err, int err_len) {
	FILE *f = fopen(path, "r");
	if(f == NULL) {
		snprintf(err, err_len, "Initial_conditions_file '%s' is not readable", path);
		return NULL;
	}
	int N;
	double box[3];
	/* header "step N Lx Ly Lz" (system.c:80-81) */
	if(fscanf(f, "%*d %d %lf %lf %lf\n", &N, box, box + 1, box + 2) != 4 || N < 0) {
		snprintf(err, err_len, "The initial configuration file '%s' is empty or its headers are malformed", path);
		fclose(f);
		return NULL;
	}
	orc_system *s = o_alloc(N, prm);
	if(s == NULL) {
		fclose(f);
		snprintf(err, err_len, "out of memory");
		return NULL;
	}
	memcpy(s->box, box, sizeof(box));
	/* three lines per particle: orientation row 0, row 1, position (system.c:213-243) */
	int i = 0;
	double p1[3] = { 0., 0., 0. }, p2[3] = { 0., 0., 0. }, p3[3], extra[3];
	char line[512];
	char *sr = fgets(line, sizeof(line), f);
	while(sr != NULL) {
		/* records beyond the header's count are only counted, for the message below (the reference writes
		 * them past its particle array) */
		double *r = i < N ? s->r + 3 * i : extra;
		/* the reference does not check these scans either: a short record keeps the previous values */
		int got = sscanf(line, "%lf %lf %lf\n", p1, p1 + 1, p1 + 2);
		got += fscanf(f, "%lf %lf %lf\n", p2, p2 + 1, p2 + 2);
		got += fscanf(f, "%lf %lf %lf\n", r, r + 1, r + 2);
		(void) got;
		if(i >= N) {
			i++;
			sr = fgets(line, sizeof(line), f);
			continue;
		}
		o_normalize(p1);
		o_normalize(p2);
		o_cross(p1, p2, p3);
		double *R = s->R + 9 * i;
		memcpy(R, p1, sizeof(p1));
		memcpy(R + 3, p2, sizeof(p2));
		memcpy(R + 6, p3, sizeof(p3));
		o_gram_schmidt(R, R + 3, R + 6);
		i++;
		sr = fgets(line, sizeof(line), f);
	}
	fclose(f);
	if(i != N) {
		snprintf(err, err_len, "Number of particles found in configuration (%d) is different from the value found in the header (%d)", i, N);
		orc_free(s);
		return NULL;
	}
	if(o_finish(s) != 0) {
		snprintf(err, err_len, "out of memory");
		orc_free(s);
		return NULL;
	}
	return s;
}

orc_system *orc_from_arrays(int N, const double *r, const double *R, const double box[3], const orc_params *prm) {
	orc_system *s = o_alloc(N, prm);
	if(s == NULL) return NULL;
	memcpy(s->box, box, 3 * sizeof(double));
	memcpy(s->r, r, 3 * sizeof(double) * N);
	memcpy(s->R, R, 9 * sizeof(double) * N);
	if(o_finish(s) != 0) {
		orc_free(s);
		return NULL;
	}
	return s;
}

void orc_free(orc_system *s) {
	if(s == NULL) return;
	free(s->sus_hist);
	free(s->r);
	free(s->r_old);
	free(s->R);
	free(s->R_old);
	free(s->patch);
	free(s->head);
	free(s->next);
	free(s->cell);
	free(s->cell_old);
	free(s->vm_links);
	free(s->vm_counter);
	free(s->vm_copies);
	free(s->vm_in);
	free(s->vm_clust);
	free(s->vm_pre);
	free(s->vm_fail);
	free(s);
}

int orc_N(const orc_system *s) { return s->N; }
void orc_box(const orc_system *s, double box[3]) { memcpy(box, s->box, 3 * sizeof(double)); }
double orc_volume(const orc_system *s) { return s->V; }
double orc_get_energy(const orc_system *s) { return s->energy; }
void orc_set_energy(orc_system *s, double E) { s->energy = E; }

void orc_get_state(const orc_system *s, double *r, double *R) {
	if(r) memcpy(r, s->r, 3 * sizeof(double) * s->N);
	if(R) memcpy(R, s->R, 9 * sizeof(double) * s->N);
}

void orc_get_patches(const orc_system *s, double *patches) { memcpy(patches, s->patch, 12 * sizeof(double) * s->N); }

void orc_counters(const orc_system *s, long long tries[ORC_N_MOVES], long long accepted[ORC_N_MOVES]) {
	memcpy(tries, s->tries, sizeof(s->tries));
	memcpy(accepted, s->accepted, sizeof(s->accepted));
}

void orc_reset_counters(orc_system *s) { /* utils_reset_acceptance_counters, utils.c:276-282 */
	memset(s->tries, 0, sizeof(s->tries));
	memset(s->accepted, 0, sizeof(s->accepted));
}

int orc_save_rrr(const orc_system *s, long long step, const char *path) { /* output_save, output.c:302-317 */
	FILE *out = fopen(path, "w");
	if(out == NULL) return -1;
	fprintf(out, "%lld %d %.12lf %.12lf %.12lf\n", step, s->N, s->box[0], s->box[1], s->box[2]);
	for(int i = 0; i < s->N; i++) {
		const double *R = s->R + 9 * i, *r = s->r + 3 * i;
		fprintf(out, "%lf %lf %lf\n", R[0], R[1], R[2]);
		fprintf(out, "%lf %lf %lf\n", R[3], R[4], R[5]);
		fprintf(out, "%.12lf %.12lf %.12lf\n", r[0], r[1], r[2]);
	}
	fclose(out);
	return 0;
}

/* ---------------------------------------------------------------- bounded multi-core throughput sample */
typedef struct {
	int N;
	const double *r, *R;
	double box[3];
	orc_params prm;
	double seconds;
	long long attempts;
	double elapsed;
	int initial_energy_ok;
} o_job;

static double o_now(void) {
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void *o_worker(void *arg) {
	o_job *j = arg;
	orc_system *s = orc_from_arrays(j->N, j->r, j->R, j->box, &j->prm);
	if(s == NULL) return NULL;
	int ov = 0;
	double E = 0.;
	for(int i = 0; i < s->N && !ov; i++) E += orc_particle_energy(s, i, &ov);
	s->energy = 0.5 * E;
	j->initial_energy_ok = !ov;
	double t0 = o_now();
	long long n = 0;
	const int chunk = 4096;
	do {
		for(int k = 0; k < chunk; k++) o_attempt(s);
		n += chunk;
	} while(o_now() - t0 < j->seconds);
	j->elapsed = o_now() - t0;
	j->attempts = n;
	orc_free(s);
	return NULL;
}

double orc_parallel_throughput(int N, const double *r, const double *R, const double box[3], const orc_params *prm,
		int threads, double seconds, long long *attempts_out) {
	if(threads < 1) threads = 1;
	o_job *jobs = calloc(threads, sizeof(o_job));
	pthread_t *tid = calloc(threads, sizeof(pthread_t));
	for(int t = 0; t < threads; t++) {
		jobs[t].N = N;
		jobs[t].r = r;
		jobs[t].R = R;
		memcpy(jobs[t].box, box, 3 * sizeof(double));
		jobs[t].prm = *prm;
		jobs[t].prm.seed = prm->seed + t;
		jobs[t].seconds = seconds;
		pthread_create(&tid[t], NULL, o_worker, &jobs[t]);
	}
	double rate = 0.;
	long long total = 0;
	for(int t = 0; t < threads; t++) {
		pthread_join(tid[t], NULL);
		if(jobs[t].elapsed > 0) rate += jobs[t].attempts / jobs[t].elapsed;
		total += jobs[t].attempts;
	}
	free(jobs);
	free(tid);
	if(attempts_out) *attempts_out = total;
	return rate;
}

/* ---------------------------------------------------------------- persistent pool */
struct orc_pool {
	int threads;
	orc_system **sys;
	double seconds;
	long long *att;
	double *el;
};

typedef struct {
	orc_pool *pool;
	int t;
} o_pool_arg;

static void *o_pool_init(void *arg) {
	o_pool_arg *a = arg;
	orc_system *s = a->pool->sys[a->t];
	int ov = 0;
	double E = 0.;
	for(int i = 0; i < s->N && !ov; i++) E += orc_particle_energy(s, i, &ov);
	s->energy = 0.5 * E;
	return NULL;
}

static void *o_pool_work(void *arg) {
	o_pool_arg *a = arg;
	orc_system *s = a->pool->sys[a->t];
	double t0 = o_now();
	long long n = 0;
	const int chunk = 4096;
	do {
		for(int k = 0; k < chunk; k++) o_attempt(s);
		n += chunk;
	} while(o_now() - t0 < a->pool->seconds);
	a->pool->el[a->t] = o_now() - t0;
	a->pool->att[a->t] = n;
	return NULL;
}

orc_pool *orc_pool_create(int N, const double *r, const double *R, const double box[3], const orc_params *prm, int threads) {
	if(threads < 1) threads = 1;
	orc_pool *p = calloc(1, sizeof(orc_pool));
	p->threads = threads;
	p->sys = calloc(threads, sizeof(orc_system *));
	p->att = calloc(threads, sizeof(long long));
	p->el = calloc(threads, sizeof(double));
	for(int t = 0; t < threads; t++) {
		orc_params q = *prm;
		q.seed = prm->seed + t;
		p->sys[t] = orc_from_arrays(N, r, R, box, &q);
		if(p->sys[t] == NULL) {
			orc_pool_free(p);
			return NULL;
		}
	}
	pthread_t *tid = calloc(threads, sizeof(pthread_t));
	o_pool_arg *args = calloc(threads, sizeof(o_pool_arg));
	for(int t = 0; t < threads; t++) {
		args[t].pool = p;
		args[t].t = t;
		pthread_create(&tid[t], NULL, o_pool_init, &args[t]);
	}
	for(int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
	free(tid);
	free(args);
	return p;
}

double orc_pool_run(orc_pool *p, double seconds, long long *attempts_out) {
	p->seconds = seconds;
	pthread_t *tid = calloc(p->threads, sizeof(pthread_t));
	o_pool_arg *args = calloc(p->threads, sizeof(o_pool_arg));
	for(int t = 0; t < p->threads; t++) {
		args[t].pool = p;
		args[t].t = t;
		pthread_create(&tid[t], NULL, o_pool_work, &args[t]);
	}
	double rate = 0.;
	long long tot = 0;
	for(int t = 0; t < p->threads; t++) {
		pthread_join(tid[t], NULL);
		if(p->el[t] > 0) rate += p->att[t] / p->el[t];
		tot += p->att[t];
	}
	free(tid);
	free(args);
	if(attempts_out) *attempts_out = tot;
	return rate;
}

void orc_pool_free(orc_pool *p) {
	if(p == NULL) return;
	for(int t = 0; t < p->threads; t++) orc_free(p->sys[t]);
	free(p->sys);
	free(p->att);
	free(p->el);
	free(p);
}
