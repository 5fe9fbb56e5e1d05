/*
 * ppgpu_cli.c -- command-line driver: runs a PatchyParticles input file (Dynamics 0, 1 or 2, Ensemble 0, 1, 3 or 5)
 * on the GB300 engine through the public C-ABI (include/ppgpu.h) and writes the reference's output files.
 *
 *   ppgpu input_file
 *
 * It follows the reference's main loop (main.c:26-143): initial energy and overlap check (main.c:55-64),
 * output_print every Print_every steps (output.c:119-211: energy.dat, density.dat, boxshape.dat,
 * acceptance.dat, the stdout line, last.rrr) with MC_check_energy after it (main.c:86), configurations
 * every Save_every steps (main.c:96-101, output.c:302-317), bond files bonds_<step>.dat with every print when
 * Print_bonds is set (output.c:206-268; partners in ascending order, where the reference lists them in
 * the order of its cell walk) and the final configuration and line
 * (main.c:125-143). The input keys are the reference's (parse_input.c: "key = value" lines, '#'
 * comments), with the same mandatory keys and error messages; the sweeps between two outputs are one
 * pp_gpu_sweeps call. Optional engine keys: GPU_resort_every (rounds between cell re-sorts),
 * GPU_neighbour_lists (1 on, 0 off), GPU_precision (0 FP32 with the FP64 guard band, 1 FP64),
 * GPU_autotune (trial sweeps of the schedule autotuner before the run; 0 = off), GPU_device.
 *
 * The Monte Carlo trajectory is the GPU checkerboard engine's, not the reference's sequential one, so only
 * the step-0 outputs coincide with the reference's line for line; the state points sampled are the same.
 */
#include "ppgpu.h"

#include <ctype.h>
#include <signal.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#define MAXKEYS 512
#define KEYLEN 512

typedef struct {
	int n;
	char key[MAXKEYS][KEYLEN];
	char val[MAXKEYS][KEYLEN];
} input_t;

static volatile sig_atomic_t g_stop = 0;
static void on_signal(int sig) {
	(void) sig;
	g_stop = 1; /* leave the main loop between two output blocks, as the reference does (main.c:15-24) */
}

/* output_exit (output.c:374-388): message on stderr, exit status 1 */
static void die(const char *fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vfprintf(stderr, fmt, ap);
	va_end(ap);
	fputc('\n', stderr);
	exit(1);
}

static void strip(char *s) {
	size_t n = strlen(s), b = 0;
	while(n > 0 && isspace((unsigned char) s[n - 1])) s[--n] = '\0';
	while(s[b] && isspace((unsigned char) s[b])) b++;
	if(b) memmove(s, s + b, strlen(s + b) + 1);
}

static void read_input(input_t *in, const char *path) {
	FILE *f = fopen(path, "r");
	if(f == NULL) die("Input file '%s' not found", path);
	char line[4 * KEYLEN];
	in->n = 0;
	while(fgets(line, sizeof(line), f)) {
		strip(line);
		if(line[0] == '\0' || line[0] == '#') continue;
		char *eq = strchr(line, '=');
		if(eq == NULL) {
			fprintf(stderr, "WARNING: malformed line '%s'\n", line); /* as loadInput does (parse_input.c:30-87) */
			continue;
		}
		if(in->n == MAXKEYS) continue;
		*eq = '\0';
		snprintf(in->key[in->n], KEYLEN, "%.*s", KEYLEN - 1, line);
		snprintf(in->val[in->n], KEYLEN, "%.*s", KEYLEN - 1, eq + 1);
		strip(in->key[in->n]);
		strip(in->val[in->n]);
		in->n++;
	}
	fclose(f);
}

/* the value of a key; a missing mandatory key stops the program (parse_input.c:97-100) */
static const char *key(const input_t *in, const char *k, int mandatory) {
	for(int i = 0; i < in->n; i++)
		if(strcmp(in->key[i], k) == 0 && in->val[i][0]) return in->val[i];
	if(mandatory) {
		fprintf(stderr, "Mandatory key '%s' not found, exiting\n", k);
		exit(-1);
	}
	return NULL;
}

static double key_d(const input_t *in, const char *k, int mandatory, double def) {
	const char *v = key(in, k, mandatory);
	return v ? atof(v) : def;
}

static long long key_ll(const input_t *in, const char *k, int mandatory, long long def) {
	const char *v = key(in, k, mandatory);
	return v ? atoll(v) : def;
}

static FILE *open_or_die(const char *name, const char *mode) {
	FILE *f = fopen(name, mode);
	if(f == NULL) die("%s is not writable", name);
	return f;
}

typedef struct {
	pp_engine *e;
	int N, ensemble, lx, avb, vmmc;
	double *r, *R, box[3]; /* room for the largest particle count the ensemble allows */
	const char *sus_folder; /* SUS: sus-<step>.dat into this folder (output.c:343-356) */
	int n_min, n_max;
	FILE *energy, *acc, *density, *boxshape;
	const char *last;
	const char *bonds_folder; /* Print_bonds: bonds_<step>.dat into this folder (output.c:88-99) */
	int *offsets, *partners, cap;
} run_t;

static void check(run_t *s, int rc) {
	if(rc == PP_OK) return;
	if(rc == PP_ERR_OVERLAP) die("\nComputing energy from scratch resulted in an overlap, aborting");
	die("%s", pp_gpu_last_error(s->e));
}

static void save(run_t *s, long long step, const char *path) {
	s->N = pp_gpu_num_particles(s->e, 0); /* GC / SUS: the current count */
	check(s, pp_gpu_download(s->e, s->r, s->R, s->box));
	if(pp_rrr_write(path, step, s->N, s->r, s->R, s->box) != PP_OK) die("Configuration file '%s' is not writable", path);
}

/* output_print_bonds (output.c:213-268): N, then per particle "index n_bonds" and its partners */
static void print_bonds(run_t *s, long long step) {
	int n = pp_gpu_bond_lists(s->e, 0, s->offsets, s->partners, s->cap);
	if(n == PP_ERR_CAPACITY && s->offsets[s->N] > s->cap) { /* the partner buffer was too small: grow it once */
		s->cap = s->offsets[s->N];
		free(s->partners);
		s->partners = malloc(sizeof(int) * (size_t) s->cap);
		if(s->partners == NULL) die("out of memory");
		n = pp_gpu_bond_lists(s->e, 0, s->offsets, s->partners, s->cap);
	}
	if(n < 0) die("%s", pp_gpu_last_error(s->e));
	char name[4 * KEYLEN];
	snprintf(name, sizeof(name), "%s/bonds_%lld.dat", s->bonds_folder, step);
	FILE *out = fopen(name, "w");
	if(out == NULL) die("Cannot create files in directory '%s'", s->bonds_folder);
	fprintf(out, "%d\n", s->N);
	for(int i = 0; i < s->N; i++) {
		fprintf(out, "%d %d\n", i, s->offsets[i + 1] - s->offsets[i]);
		for(int k = s->offsets[i]; k < s->offsets[i + 1]; k++) fprintf(out, "%d ", s->partners[k]);
		fprintf(out, "\n");
	}
	fclose(out);
}

/* output_print (output.c:119-211) */
static void print_step(run_t *s, long long step) {
	double energy = 0.;
	pp_counters c;
	check(s, pp_gpu_get_energy(s->e, 0, &energy));
	check(s, pp_gpu_counters(s->e, 0, &c, 1));
	check(s, pp_gpu_box(s->e, 0, s->box));
	s->N = pp_gpu_num_particles(s->e, 0);
	const double V = s->box[0] * s->box[1] * s->box[2], E = s->N > 0 ? energy / s->N : 0.;
	fprintf(s->energy, "%lld %lf\n", step, E);
	fflush(s->energy);
	if(s->ensemble != PP_NVT) {
		fprintf(s->density, "%lld %lf %d\n", step, s->N / V, s->N);
		fflush(s->density);
	}
	if(s->lx) {
		fprintf(s->boxshape, "%lld %lf %lf %lf\n", step, s->box[0], s->box[1], s->box[2]);
		fflush(s->boxshape);
	}
	/* output.c:149-162: the dynamics' columns */
	if(s->vmmc) fprintf(s->acc, "%lld %e", step, c.accepted[PP_MOVE_VMMC] / (double) c.tries[PP_MOVE_VMMC]);
	else fprintf(s->acc, "%lld %e", step, c.accepted[PP_MOVE_ROTO_TRASL] / (double) c.tries[PP_MOVE_ROTO_TRASL]);
	if(s->avb) fprintf(s->acc, " %e", c.accepted[PP_MOVE_AVB] / (double) c.tries[PP_MOVE_AVB]);
	if(s->ensemble == PP_GC || s->ensemble == PP_SUS) {
		fprintf(s->acc, " %e", c.accepted[PP_MOVE_ADD] / (double) c.tries[PP_MOVE_ADD]);
		fprintf(s->acc, " %e", c.accepted[PP_MOVE_REMOVE] / (double) c.tries[PP_MOVE_REMOVE]);
	}
	if(s->ensemble == PP_NPT) fprintf(s->acc, " %e", c.accepted[PP_MOVE_VOLUME] / (double) c.tries[PP_MOVE_VOLUME]);
	if(s->lx) fprintf(s->acc, " %e", c.accepted[PP_MOVE_LX] / (double) c.tries[PP_MOVE_LX]);
	fprintf(s->acc, "\n");
	fflush(s->acc);
	printf("%lld %lf %lf", step, E, energy);
	if(s->ensemble != PP_NVT) printf(" %lf", s->N / V);
	printf("\n");
	fflush(stdout);
	save(s, step, s->last);
	if(s->bonds_folder) print_bonds(s, step);
}

int main(int argc, char *argv[]) {
	if(argc < 2) die("Usage is %s input", argv[0]);
	signal(SIGTERM, on_signal);
	signal(SIGINT, on_signal);
	signal(SIGUSR2, on_signal);
	input_t *in = calloc(1, sizeof(input_t));
	if(in == NULL) die("out of memory");
	read_input(in, argv[1]);

	/* output_init (output.c:19-109) */
	const char *v;
	const int restart = (v = key(in, "Restart_step_counter", 0)) ? atoi(v) : 1;
	const char *mode = restart ? "w" : "a";
	const char *conf = key(in, "Initial_conditions_file", 1);
	long long start_from = 0, step0 = 0;
	int N = 0;
	run_t s;
	memset(&s, 0, sizeof(s));
	if(pp_rrr_header(conf, &step0, &N, s.box) != PP_OK) die("Initial configuration file '%s' not found or unreadable", conf);
	if(!restart) start_from = step0;
	const long long print_every = key_ll(in, "Print_every", 1, 0), save_every = key_ll(in, "Save_every", 1, 0);
	if(print_every <= 0 || save_every <= 0) die("Print_every and Save_every must be positive");
	s.energy = open_or_die((v = key(in, "Energy_file", 0)) ? v : "energy.dat", mode);
	s.acc = open_or_die((v = key(in, "Acceptance_file", 0)) ? v : "acceptance.dat", mode);
	const char *folder = key(in, "Configuration_folder", 1);
	if(access(folder, W_OK) != 0) die("Cannot create files in directory '%s': please make sure that the directory exists and it is writable", folder);
	s.last = (v = key(in, "Configuration_last", 0)) ? v : "last.rrr";
	if((v = key(in, "Print_bonds", 0)) && atoi(v)) {
		s.bonds_folder = key(in, "Bonds_folder", 1);
		if(access(s.bonds_folder, W_OK) != 0)
			die("Cannot create files in directory '%s': please make sure that the directory exists and it is writable", s.bonds_folder);
	}

	/* system_init (system.c:58-252) and MC_init (MC.c:85-131) */
	pp_params p;
	pp_default_params(&p);
	const int dynamics = (int) key_ll(in, "Dynamics", 1, 0);
	s.ensemble = p.ensemble = (int) key_ll(in, "Ensemble", 1, 0);
	if(dynamics != PP_RTMC && dynamics != PP_VMMC && dynamics != PP_AVBMC)
		die("Dynamics = %d is not run by this engine (0 roto-translations, 1 VMMC, 2 AVB moves and roto-translations)", dynamics);
	p.dynamics = dynamics;
	if(dynamics == PP_VMMC) { /* VMMC_init (vmmc.c:15-45): both keys mandatory */
		s.vmmc = 1;
		p.vmmc_max_move = key_d(in, "vmmc_max_move", 1, 0.);
		p.vmmc_max_cluster = (int) key_ll(in, "vmmc_max_cluster", 1, 0);
	}
	if(dynamics == PP_AVBMC) { /* AVBMC_init (avb.c:13-36): the optional avb_p */
		s.avb = 1;
		p.avb_p = key_d(in, "avb_p", 0, 0.5);
	}
	if(s.ensemble != PP_NVT && s.ensemble != PP_NPT && s.ensemble != PP_GC && s.ensemble != PP_SUS)
		die("Ensemble = %d is not run by this engine (0 NVT, 1 GC, 3 SUS, 5 NPT)", s.ensemble);
	if(s.ensemble != PP_NVT) s.density = open_or_die((v = key(in, "Density_file", 0)) ? v : "density.dat", mode);
	if(s.bonds_folder && s.ensemble != PP_NVT) die("The printing of bonds is unavailable in non-canonical ensembles"); /* output.c:90-92 */
	if(s.ensemble == PP_SUS) { /* output.c:79-84 */
		s.sus_folder = key(in, "Umbrella_sampling_folder", 1);
		if(access(s.sus_folder, W_OK) != 0)
			die("Cannot create files in directory '%s': please make sure that the directory exists and it is writable", s.sus_folder);
	}
	if(s.ensemble == PP_GC || s.ensemble == PP_SUS) { /* system.c:90-103 */
		p.activity = key_d(in, "Activity", 1, 0.);
		if(s.ensemble == PP_GC) p.n_max = (int) key_ll(in, "GC_N_max", 1, 0);
		else {
			p.n_min = (int) key_ll(in, "Umbrella_sampling_min", 1, 0);
			p.n_max = (int) key_ll(in, "Umbrella_sampling_max", 1, 0);
		}
		s.n_min = p.n_min;
		s.n_max = p.n_max;
	}
	p.disp_max = key_d(in, "Disp_max", 1, 0.);
	p.theta_max = key_d(in, "Theta_max", 1, 0.);
	p.temperature = key_d(in, "Temperature", 1, 0.);
	if((v = key(in, "Seed", 0))) p.seed = (uint64_t) (long long) atoll(v);
	else {
		p.seed = (uint64_t) time(NULL);
		fprintf(stderr, "Using seed %llu\n", (unsigned long long) p.seed);
	}
	p.kf_delta = key_d(in, "KF_delta", 1, 0.);
	p.kf_cosmax = key_d(in, "KF_cosmax", 1, 0.);
	if(s.ensemble == PP_NPT) {
		p.rescale_factor_max = key_d(in, "rescale_factor_max", 1, 0.);
		p.pressure = key_d(in, "P", 1, 0.);
	}
	else if((v = key(in, "Lx_move", 0)) && atoi(v)) {
		p.lx_move = atoi(v) == 2 ? 2 : 1;
		p.lx_change_max = key_d(in, "Lx_change_max", 1, 0.);
		p.lyz_min = key_d(in, "Lyz_min", 1, 0.);
		p.lyz_max = key_d(in, "Lyz_max", 1, 0.);
		s.lx = 1;
	}
	if((v = key(in, "Lx_move", 0)) && atoi(v)) s.boxshape = open_or_die("boxshape.dat", mode); /* output.c:101-108 */
	p.resort_every = (int) key_ll(in, "GPU_resort_every", 0, 0);
	p.precision = (int) key_ll(in, "GPU_precision", 0, PP_PREC_FP32_GUARD);
	if((v = key(in, "GPU_device", 0)) && pp_gpu_select_device(atoi(v)) != PP_OK) die("cannot select GPU %s", v);

	const int room = (N > s.n_max ? N : s.n_max) > 0 ? (N > s.n_max ? N : s.n_max) : 1;
	s.r = malloc(sizeof(double) * 3 * (size_t) room);
	s.R = malloc(sizeof(double) * 9 * (size_t) room);
	if(s.r == NULL || s.R == NULL) die("out of memory");
	char err[512];
	if(pp_rrr_read(conf, N, s.r, s.R, s.box, err, sizeof(err)) != PP_OK) die("%s", err);
	s.N = N;
	s.cap = 8 * (N > 0 ? N : 1);
	s.offsets = calloc((size_t) N + 1, sizeof(int));
	s.partners = malloc(sizeof(int) * (size_t) s.cap);
	if(s.offsets == NULL || s.partners == NULL) die("out of memory");
	if(pp_gpu_create(&p, &s.e) != PP_OK) die("%s", pp_gpu_last_error(s.e));
	if((v = key(in, "GPU_neighbour_lists", 0))) check(&s, pp_gpu_set_neighbour_lists(s.e, atoi(v)));
	/* the upload computes the initial energy and refuses an overlapping configuration (main.c:55-64) */
	const int rc = pp_gpu_upload(s.e, N, s.r, s.R, s.box);
	if(rc == PP_ERR_OVERLAP) die("Initial configuration contains an overlap, aborting");
	if(rc != PP_OK) die("%s", pp_gpu_last_error(s.e));
	double energy = 0.;
	check(&s, pp_gpu_get_energy(s.e, 0, &energy));
	fprintf(stderr, "Initial energy: %lf\n", N > 0 ? energy / N : 0.);
	if((v = key(in, "GPU_autotune", 0)) && atoi(v) > 0) {
		pp_tune_result t;
		check(&s, pp_gpu_autotune(s.e, atoi(v), &t));
		check(&s, pp_gpu_counters(s.e, 0, NULL, 1)); /* the trial sweeps are not part of the reported run */
		fprintf(stderr, "Schedule: resort_every %d, reorder_every %d, cell_scale %.2f, neighbour lists %d (%.3g attempts/s)\n", t.resort_every,
				t.reorder_every, t.cell_scale, t.neighbour_lists, t.attempts_per_s);
	}

	/* main loop (main.c:78-120): the sweeps between two output steps are one pp_gpu_sweeps call */
	const long long steps = key_ll(in, "Steps", 1, 0) + start_from;
	long long step = start_from;
	char name[4 * KEYLEN];
	while(step < steps && !g_stop) {
		if(step % print_every == 0) {
			print_step(&s, step);
			if(step != 0) {
				check(&s, pp_gpu_check_energy(s.e, 0)); /* MC_check_energy (main.c:86) */
				if(s.ensemble == PP_SUS) { /* output_and_reset_sus (main.c:89, output.c:343-356) */
					const int nb = s.n_max - s.n_min + 1;
					long long *h = malloc(sizeof(long long) * (size_t) nb);
					if(h == NULL) die("out of memory");
					check(&s, pp_gpu_sus_histogram(s.e, h, 1));
					snprintf(name, sizeof(name), "%s/sus-%lld.dat", s.sus_folder, step);
					FILE *fs = fopen(name, "w");
					if(fs == NULL) die("SUS file '%s' is not writable", name);
					for(int b = 0; b < nb; b++)
						if(h[b] > 0) fprintf(fs, "%d %lld\n", b + s.n_min, h[b]);
					fclose(fs);
					free(h);
				}
			}
		}
		if(step > 0 && step % save_every == 0) {
			snprintf(name, sizeof(name), "%s/conf_%lld.rrr", folder, step);
			save(&s, step, name);
			save(&s, step, s.last);
		}
		long long next = steps;
		const long long np = (step / print_every + 1) * print_every, ns = (step / save_every + 1) * save_every;
		if(np < next) next = np;
		if(ns < next) next = ns;
		check(&s, pp_gpu_sweeps(s.e, next - step));
		step = next;
	}
	save(&s, step, s.last);
	check(&s, pp_gpu_get_energy(s.e, 0, &energy));
	check(&s, pp_gpu_box(s.e, 0, s.box));
	N = s.N;
	printf("%lld %lf %lf", step, N > 0 ? energy / N : 0., energy);
	if(s.ensemble != PP_NVT) printf(" %lf", N / (s.box[0] * s.box[1] * s.box[2]));
	printf("\n");
	fclose(s.energy);
	fclose(s.acc);
	if(s.density) fclose(s.density);
	if(s.boxshape) fclose(s.boxshape);
	pp_gpu_destroy(s.e);
	free(s.r);
	free(s.R);
	free(s.offsets);
	free(s.partners);
	free(in);
	return 0;
}
