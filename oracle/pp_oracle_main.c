/*
 * pp_oracle_main.c -- TEST INFRASTRUCTURE: command-line driver of the oracle restatement, mirroring the
 * reference main loop (main.c:26-143) for Dynamics = 0 in the NVT, NPT, GC and SUS ensembles, with the reference
 * input-file rules (parse_input.c:18-104) and output files (output.c:19-211, 302-317). Used to show that
 * the restatement reproduces the reference trajectory: same input file -> same energy.dat,
 * acceptance.dat, density.dat, stdout and configuration files.
 *
 *   pporacle input_file
 */
#include "pp_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define MAXKEYS 256
#define KEYLEN 256

typedef struct {
	int n;
	char key[MAXKEYS][KEYLEN];
	char val[MAXKEYS][KEYLEN];
} inp_t;

static void trim(char *s) {
	size_t n = strlen(s);
	while(n > 0 && isspace((unsigned char) s[n - 1])) s[--n] = '\0';
	size_t b = 0;
	while(s[b] && isspace((unsigned char) s[b])) b++;
	if(b) memmove(s, s + b, strlen(s + b) + 1);
}

/* a key or value cut to the table's fixed width (the reference's OPT_MAX_LENGTH strings, parse_input.h:16) */
static void copy_field(char *dst, const char *src) {
	size_t n = strlen(src);
	if(n >= KEYLEN) n = KEYLEN - 1;
	memcpy(dst, src, n);
	dst[n] = '\0';
}

/* loadInput (parse_input.c:30-87): "key = value" lines, '#' comments, surrounding blanks trimmed */
static int load_input(inp_t *in, const char *path) {
	FILE *f = fopen(path, "r");
	if(f == NULL) {
		fprintf(stderr, "Input file not found\n");
		return -1;
	}
	in->n = 0;
	char line[4096];
	while(fgets(line, sizeof(line), f)) {
		trim(line);
		if(line[0] == '\0' || line[0] == '#') continue;
		char *eq = strchr(line, '=');
		if(eq == NULL) {
			fprintf(stderr, "WARNING: malformed line '%s'\n", line);
			continue;
		}
		*eq = '\0';
		if(in->n == MAXKEYS) break;
		copy_field(in->key[in->n], line);
		copy_field(in->val[in->n], eq + 1);
		trim(in->key[in->n]);
		trim(in->val[in->n]);
		in->n++;
	}
	fclose(f);
	return 0;
}

/* getInputKeyIndex (parse_input.c:89-104): first key with a non-empty value; missing mandatory -> exit(-1) */
static const char *get(inp_t *in, const char *key, int mandatory) {
	for(int i = 0; i < in->n; i++)
		if(strcmp(in->key[i], key) == 0 && strlen(in->val[i]) > 0) return in->val[i];
	if(mandatory) {
		fprintf(stderr, "Mandatory key '%s' not found, exiting\n", key);
		exit(-1);
	}
	return NULL;
}

static void die(const char *msg) {
	fprintf(stderr, "%s\n", msg);
	exit(1);
}

int main(int argc, char *argv[]) {
	if(argc < 2) {
		fprintf(stderr, "Usage is %s input\n", argv[0]);
		return 1;
	}
	inp_t *in = calloc(1, sizeof(inp_t));
	if(load_input(in, argv[1]) != 0) return 1;

	/* output_init (output.c:19-109), the parts that Dynamics = 0 with NVT/NPT reads */
	int restart = 1;
	const char *v;
	if((v = get(in, "Restart_step_counter", 0))) restart = atoi(v);
	const char *mode = restart ? "w" : "a";
	long long start_from = 0;
	if(!restart) {
		FILE *c = fopen(get(in, "Initial_conditions_file", 1), "r");
		if(c == NULL || fscanf(c, "%lld", &start_from) != 1) die("Invalid initial configuration: the first value in the first row should be the time step of the configuration");
		fclose(c);
	}
	long long print_every = atol(get(in, "Print_every", 1));
	long long save_every = atol(get(in, "Save_every", 1));
	const char *ename = (v = get(in, "Energy_file", 0)) ? v : "energy.dat";
	const char *aname = (v = get(in, "Acceptance_file", 0)) ? v : "acceptance.dat";
	FILE *fe = fopen(ename, mode), *fa = fopen(aname, mode), *fd = NULL;
	if(fe == NULL || fa == NULL) die("output file not writable");
	const char *folder = get(in, "Configuration_folder", 1);
	if(access(folder, W_OK) != 0) die("Cannot create files in the configuration folder");
	const char *last = (v = get(in, "Configuration_last", 0)) ? v : "last.rrr";
	int ensemble = atoi(get(in, "Ensemble", 1));
	const char *sus_folder = NULL;
	if(ensemble != 0) {
		const char *dname = (v = get(in, "Density_file", 0)) ? v : "density.dat";
		fd = fopen(dname, mode);
		if(fd == NULL) die("Density file not writable");
		if(ensemble == ORC_SUS) { /* output.c:79-84 */
			sus_folder = get(in, "Umbrella_sampling_folder", 1);
			if(access(sus_folder, W_OK) != 0) die("Cannot create files in the umbrella sampling folder");
		}
	}

	/* system_init (system.c:58-252), Dynamics = 0 or 2 */
	orc_params prm;
	memset(&prm, 0, sizeof(prm));
	int dynamics = atoi(get(in, "Dynamics", 1));
	prm.ensemble = ensemble;
	prm.dynamics = dynamics;
	if(dynamics == ORC_AVBMC && (v = get(in, "avb_p", 0))) prm.avb_p = atof(v); /* avb.c:35 */
	prm.disp_max = atof(get(in, "Disp_max", 1));
	prm.theta_max = atof(get(in, "Theta_max", 1));
	prm.T = atof(get(in, "Temperature", 1));
	const char *conf = get(in, "Initial_conditions_file", 1);
	if(!(v = get(in, "Seed", 0))) die("this driver needs an explicit Seed");
	prm.seed = atoi(v);
	prm.kf_delta = atof(get(in, "KF_delta", 1));
	prm.kf_cosmax = atof(get(in, "KF_cosmax", 1));
	if(ensemble == ORC_GC || ensemble == ORC_SUS) { /* system.c:90-103 */
		prm.activity = atof(get(in, "Activity", 1));
		if(ensemble == ORC_GC) prm.n_max = atoi(get(in, "GC_N_max", 1));
		else {
			prm.n_min = atoi(get(in, "Umbrella_sampling_min", 1));
			prm.n_max = atoi(get(in, "Umbrella_sampling_max", 1));
		}
	}
	if(ensemble == ORC_NPT) {
		prm.rescale_factor_max = atof(get(in, "rescale_factor_max", 1));
		prm.P = atof(get(in, "P", 1));
	}
	else if((v = get(in, "Lx_move", 0)) && atoi(v)) { /* system.c:170-196 (NVT only) */
		prm.lx_move = 1;
		prm.lx_change_max = atof(get(in, "Lx_change_max", 1));
		prm.lyz_min = atof(get(in, "Lyz_min", 1));
		prm.lyz_max = atof(get(in, "Lyz_max", 1));
	}
	/* boxshape.dat is opened whenever the Lx_move key is set (output.c:101-108) */
	FILE *fb = NULL;
	if((v = get(in, "Lx_move", 0)) && atoi(v)) {
		fb = fopen("boxshape.dat", mode);
		if(fb == NULL) die("boxshape.dat is not writable");
	}
	if(dynamics == ORC_VMMC) { /* VMMC_init (vmmc.c:15-45): both keys are mandatory; vmmc_max_move is read, not used */
		const double max_move = atof(get(in, "vmmc_max_move", 1));
		prm.vmmc_max_cluster = atoi(get(in, "vmmc_max_cluster", 1));
		fprintf(stderr, "Using VMMC dynamics with max_move = %lf, max_clust = %d\n", max_move, prm.vmmc_max_cluster); /* output_log_msg */
	}
	if((dynamics != ORC_RTMC && dynamics != ORC_AVBMC && dynamics != ORC_VMMC) ||
			(ensemble != ORC_NVT && ensemble != ORC_NPT && ensemble != ORC_GC && ensemble != ORC_SUS))
		die("only Dynamics = 0, 1 or 2 with Ensemble 0, 1, 3 or 5 is restated");
	char err[512];
	orc_system *s = orc_load_rrr(conf, &prm, err, sizeof(err));
	if(s == NULL) die(err);
	if(dynamics == ORC_AVBMC) { /* AVBMC_init (avb.c:13-31) */
		if(orc_avb_status(s) != 0) die("The AVB move cannot be used with patches that do not fulfill the single-bond-per-patch condition");
		double vin, vout;
		orc_avb_volumes(s, &vin, &vout);
		fprintf(stderr, "Vavb = %lf\n", vin); /* output_log_msg */
	}
	if(ensemble == ORC_SUS) { /* system.c:100-101 */
		char m[256];
		if(orc_N(s) < prm.n_min) {
			snprintf(m, sizeof(m), "Number of particles %d is smaller than Umbrella_sampling_min (%d)", orc_N(s), prm.n_min);
			die(m);
		}
		if(orc_N(s) > prm.n_max) {
			snprintf(m, sizeof(m), "Number of particles %d is larger than Umbrella_sampling_max (%d)", orc_N(s), prm.n_max);
			die(m);
		}
	}
	if(prm.lx_move) {
		double b[3];
		orc_box(s, b);
		if(b[1] != b[2]) die("Lx_move = 1 requires Ly = Lz");
		if(prm.lyz_min >= b[1]) die("Lyz_min should be smaller than box size");
		if(prm.lyz_max <= b[1]) die("Lyz_max should be larger than box size");
		fprintf(stderr, "Ly and Lz are allowed to vary between %lf and %lf\n", prm.lyz_min, prm.lyz_max); /* output_log_msg */
	}

	/* initial energy and overlap check (main.c:55-64) */
	int N = orc_N(s), ov;
	double E0 = 0.;
	for(int i = 0; i < N; i++) {
		E0 += orc_particle_energy(s, i, &ov);
		if(ov) die("Initial configuration contains an overlap, aborting");
	}
	orc_set_energy(s, 0.5 * E0);

	long long steps = atol(get(in, "Steps", 1)) + start_from, step;
	long long tries[ORC_N_MOVES], acc[ORC_N_MOVES];
	char name[1100];
	for(step = start_from; step < steps; step++) {
		N = orc_N(s);
		if(step % print_every == 0) { /* output_print (output.c:119-211) */
			double energy = orc_get_energy(s);
			double E = N > 0 ? energy / N : 0;
			double V = orc_volume(s);
			fprintf(fe, "%lld %lf\n", step, E);
			fflush(fe);
			if(ensemble != 0) {
				fprintf(fd, "%lld %lf %d\n", step, N / V, N);
				fflush(fd);
			}
			if(prm.lx_move) {
				double b[3];
				orc_box(s, b);
				fprintf(fb, "%lld %lf %lf %lf\n", step, b[0], b[1], b[2]);
				fflush(fb);
			}
			orc_counters(s, tries, acc);
			fprintf(fa, "%lld", step);
			/* output.c:149-162 */
			if(dynamics == ORC_VMMC) fprintf(fa, " %e", acc[ORC_MOVE_VMMC] / (double) tries[ORC_MOVE_VMMC]);
			else fprintf(fa, " %e", acc[ORC_ROTO_TRASL] / (double) tries[ORC_ROTO_TRASL]);
			if(dynamics == ORC_AVBMC) fprintf(fa, " %e", acc[ORC_AVB] / (double) tries[ORC_AVB]);
			if(ensemble == ORC_GC || ensemble == ORC_SUS) {
				fprintf(fa, " %e", acc[ORC_ADD] / (double) tries[ORC_ADD]);
				fprintf(fa, " %e", acc[ORC_REMOVE] / (double) tries[ORC_REMOVE]);
			}
			if(ensemble == ORC_NPT) fprintf(fa, " %e", acc[ORC_VOLUME] / (double) tries[ORC_VOLUME]);
			if(prm.lx_move) fprintf(fa, " %e", acc[ORC_LX] / (double) tries[ORC_LX]);
			fprintf(fa, "\n");
			fflush(fa);
			orc_reset_counters(s);
			printf("%lld %lf %lf", step, E, energy);
			if(ensemble != 0) printf(" %lf", N / V);
			printf("\n");
			orc_save_rrr(s, step, last);
			if(step != 0) {
				int rc = orc_check_energy(s);
				if(rc == -1) die("\nComputing energy from scratch resulted in an overlap, aborting");
				if(rc == -2) die("\nEnergy check failed");
				if(ensemble == ORC_SUS) { /* output_and_reset_sus (output.c:343-356) */
					long long h[4096];
					const int nb = orc_sus_hist(s, NULL, 0);
					if(nb > 4096) die("SUS window too wide for this driver");
					orc_sus_hist(s, h, 1);
					snprintf(name, sizeof(name), "%s/sus-%lld.dat", sus_folder, step);
					FILE *fs = fopen(name, "w");
					if(fs == NULL) die("SUS file not writable");
					for(int b = 0; b < nb; b++)
						if(h[b] > 0) fprintf(fs, "%d %lld\n", b + prm.n_min, h[b]);
					fclose(fs);
				}
			}
		}
		if(step > 0 && step % save_every == 0) {
			snprintf(name, sizeof(name), "%s/conf_%lld.rrr", folder, step);
			orc_save_rrr(s, step, name);
			orc_save_rrr(s, step, last);
		}
		orc_sweep(s);
		if(orc_vmmc_error(s)) die("VMMC: memory exhausted, or a cluster move into an overlap");
		if(orc_error(s)) { /* MC_add_remove's output_exit */
			fprintf(stderr, "The system contains the maximum number of particles set in the input file (%d), increase GC_N_max\n", prm.n_max);
			exit(1);
		}
	}
	N = orc_N(s);
	orc_save_rrr(s, step, last);
	double energy = orc_get_energy(s);
	printf("%lld %lf %lf", step, N > 0 ? energy / N : 0, energy);
	if(ensemble != 0) printf(" %lf", N / orc_volume(s));
	printf("\n");
	fclose(fe);
	fclose(fa);
	if(fd) fclose(fd);
	if(fb) fclose(fb);
	orc_free(s);
	free(in);
	return 0;
}
