/*
 * pp_oracle.h -- CPU restatement of the PatchyParticles roto-translation Monte Carlo path
 * (Kern-Frenkel four-patch hard spheres, Dynamics = 0, NVT and NPT).
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library; the product never links, imports or calls it. It is what the CUDA path is
 * compared with, and it is itself pinned against the reference compiled from source (oracle/_ref) and
 * against golden outputs of that build committed under tests/golden/.
 *
 * Every function restates one reference routine (cited file:line, paths inside the reference project)
 * with the same floating-point operation order, and the library is compiled with -ffp-contract=off,
 * so that, given the same input and seed, it reproduces the reference trajectory bit for bit.
 * Random numbers come from the POSIX drand48 recurrence implemented here per system (seeded exactly as
 * srand48 does), so several independent systems can live in one process and in several threads.
 */
#ifndef PP_ORACLE_H_
#define PP_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_OVERLAP -1
#define ORC_NO_BOND 0
#define ORC_PATCH_BOND 1

#define ORC_NVT 0
#define ORC_GC 1  /* grand canonical (defs.h:22), do_GC (MC.c:31-43) */
#define ORC_SUS 3 /* successive umbrella sampling (defs.h:23), do_SUS (MC.c:45-58) */
#define ORC_NPT 5

/* Dynamics (defs.h:27-29) */
#define ORC_RTMC 0
#define ORC_VMMC 1  /* virtual-move Monte Carlo cluster moves, vmmc.c:258-483 */
#define ORC_AVBMC 2 /* aggregation-volume-bias moves mixed with roto-translations, avb.c:77-186 */

/* move-type slots of the tries/accepted counters, as in defs.h:11-19 */
#define ORC_ROTO_TRASL 0
#define ORC_AVB 1    /* defs.h:13 */
#define ORC_ADD 2    /* defs.h:14 */
#define ORC_REMOVE 3 /* defs.h:15 */
#define ORC_MOVE_VMMC 5 /* defs.h:17 */
#define ORC_VOLUME 6
#define ORC_LX 7 /* defs.h:19 */
#define ORC_N_MOVES 8

typedef struct orc_params {
	int ensemble;              /* ORC_NVT or ORC_NPT (defs.h:21-25) */
	double T;                  /* Temperature */
	double P;                  /* P (NPT only) */
	double disp_max;           /* Disp_max */
	double theta_max;          /* Theta_max */
	double rescale_factor_max; /* rescale_factor_max (NPT only) */
	double kf_delta;           /* KF_delta */
	double kf_cosmax;          /* KF_cosmax */
	int seed;                  /* Seed (srand48 argument, system.c:71-75) */
	int lx_move;               /* Lx_move (NVT only, system.c:165-196) */
	double lx_change_max;      /* Lx_change_max */
	double lyz_min, lyz_max;   /* Lyz_min, Lyz_max */
	double activity;           /* Activity z (GC and SUS, system.c:91) */
	int n_min, n_max;          /* GC: 0 and GC_N_max; SUS: Umbrella_sampling_min / _max (system.c:92-103) */
	int dynamics;              /* Dynamics: ORC_RTMC or ORC_AVBMC (system.c:63, MC.c:115-130) */
	double avb_p;              /* avb_p: probability of a roto-translation in AVBMC (avb.c:33-35); <= 0 selects 0.5 */
	int vmmc_max_cluster;      /* vmmc_max_cluster (vmmc.c:25): a cluster that reaches it is rejected */
} orc_params;

typedef struct orc_system orc_system;

/* Loads a .rrr configuration (system.c:77-245 reading rules). Returns NULL and fills err on failure. */
orc_system *orc_load_rrr(const char *path, const orc_params *prm, char *err, int err_len);
/* Builds a system from arrays: r is N x 3, R is N x 9 row-major orientation (already orthonormal). */
orc_system *orc_from_arrays(int N, const double *r, const double *R, const double box[3], const orc_params *prm);
void orc_free(orc_system *s);

int orc_N(const orc_system *s);
void orc_box(const orc_system *s, double box[3]);
/* syst->V: updated only by accepted volume moves (MC.c:500), as the density output uses it */
double orc_volume(const orc_system *s);
double orc_get_energy(const orc_system *s);
void orc_set_energy(orc_system *s, double E);
void orc_get_state(const orc_system *s, double *r, double *R);
void orc_get_patches(const orc_system *s, double *patches); /* N x 4 x 3 */
void orc_base_patches(double base[4][3]);
void orc_counters(const orc_system *s, long long tries[ORC_N_MOVES], long long accepted[ORC_N_MOVES]);
void orc_reset_counters(orc_system *s);

/* Pair test of particle i against particle j (MC_interact, MC.c:268-270 -> MC.c:232-266). */
int orc_interact(orc_system *s, int i, int j);
/* MC_energy of particle i (MC.c:272-309); *overlap receives syst->overlap. */
double orc_particle_energy(orc_system *s, int i, int *overlap);
/* Per-particle energies/overlap flags and full bond/overlap partner counts (27-cell walk, no early exit).
 * Returns 0.5 * sum of energies (main.c:55-64). Any output pointer may be NULL. */
double orc_energies(orc_system *s, double *E, int *overlap, int *n_bonds, int *n_overlaps);
/* Bonded partner lists: offsets (N+1) and partners (capacity cap). Returns total or -1 if cap too small. */
int orc_bond_lists(orc_system *s, int *offsets, int *partners, int cap);

/* One Monte Carlo step of the ensemble: do_NVT (MC.c:19-29), do_GC (MC.c:31-43), do_SUS (MC.c:45-58) or
 * do_NPT (MC.c:60-68). GC and SUS systems hold up to n_max particles; orc_N is the current count. */
void orc_sweep(orc_system *s);
void orc_sweeps(orc_system *s, long long n);
/* MC_check_energy (MC.c:766-784). Returns 0, -1 (overlap found) or -2 (energy drift > 1e-5). */
int orc_check_energy(orc_system *s);
/* output_save (output.c:302-317). Returns 0 or -1. */
int orc_save_rrr(const orc_system *s, long long step, const char *path);

/* The reference generator's random sequential insertion (generator.c:43-68, 99-105) with srand48(seed):
 * r (N x 3), R (N x 9 rows) and the cubic box, unrounded (generated.rrr holds them printed with %lf /
 * %.12lf). Returns 0, or -1 for a density outside (0, 0.7] or no memory. */
int orc_generate(int N, double density, int seed, double *r, double *R, double box[3]);

/* VMMC: 1 once a move ran out of link memory ("VMMC: memory exhausted", vmmc.c:176) or moved a cluster
 * into an overlap (the reference's assert, vmmc.c:436-446); the oracle then makes no further move */
int orc_vmmc_error(const orc_system *s);

/* 1 once a GC insertion found the system full (the reference stops there: "increase GC_N_max",
 * MC.c:346-348; the oracle makes no further move), else 0. */
int orc_error(const orc_system *s);
/* SUS histogram of N after every insertion/removal attempt (MC.c:50), bins N_min..N_max; reset = 1 clears
 * it as output_and_reset_sus does (output.c:343-356). Returns the number of bins. */
int orc_sus_hist(orc_system *s, long long *out, int reset);

/* AVBMC: 0, or -1 where AVBMC_init refuses the patch geometry (avb.c:14-17: the single-bond-per-patch
 * condition). A refused system makes no moves. */
int orc_avb_status(const orc_system *s);
/* AVBMC_init's bonding and non-bonding volumes (avb.c:26-28) */
void orc_avb_volumes(const orc_system *s, double *v_in, double *v_out);

/* drand48 recurrence check: n draws from a generator seeded as srand48(seed) would be. */
void orc_drand48_sequence(int seed, int n, double *out);

/* Aggregate throughput of independent systems, one per thread (bounded CPU baseline sample).
 * Each thread t clones the given arrays, seeds with seed+t and runs sweeps until `seconds` have
 * passed (at least one sweep). Returns attempts per second summed over threads; *attempts_out gets the
 * total number of attempts performed. */
double orc_parallel_throughput(int N, const double *r, const double *R, const double box[3], const orc_params *prm,
		int threads, double seconds, long long *attempts_out);

/* Persistent pool for repeated bounded samples: `threads` independent clones (seeds seed+t), initial
 * energy computed once; each orc_pool_run lets every clone continue for `seconds` and returns the
 * aggregate attempts per second of that interval. */
typedef struct orc_pool orc_pool;
orc_pool *orc_pool_create(int N, const double *r, const double *R, const double box[3], const orc_params *prm, int threads);
double orc_pool_run(orc_pool *pool, double seconds, long long *attempts_out);
void orc_pool_free(orc_pool *pool);

#ifdef __cplusplus
}
#endif

#endif /* PP_ORACLE_H_ */
