/*
 * ppgpu.h -- C-ABI of the GB300 roto-translation Monte Carlo engine for Kern-Frenkel four-patch hard
 * spheres (PatchyParticles, Dynamics = 0, NVT and NPT).
 *
 * The boundary is the reference's per-step ensemble hook: `System::do_ensemble` (defs.h:78), selected by
 * MC_init (MC.c:85-131) and called once per MC step from the driver loop (main.c:119). One engine call
 * `pp_gpu_sweeps(e, n)` replaces n calls of do_NVT (MC.c:19-29) or do_NPT (MC.c:60-68) with
 * MC_move_rototranslate (MC.c:311-340) as do_dynamics. Host <-> device traffic happens only where the
 * reference driver needs host state: the print/save cadence (main.c:82-104, output.c:119-211).
 *
 * Plain C types only: no CUDA or torch types cross this boundary. Every function returns PP_OK (0) or a
 * negative PP_ERR_* code and never exits the process; pp_gpu_last_error gives the message. The
 * reference's fatal paths (output_exit, output.c:374-388) become these codes; the command-line driver
 * maps them back to exit(1).
 *
 * Particle state crosses the boundary as the reference stores it (defs.h:47-56): positions r as N x 3
 * doubles (unwrapped, as MC_rototraslate_particle leaves them, MC.c:213-215) and orientations R as N x 9
 * doubles, row-major, rows = the three rows of PatchyParticle::orientation.
 */
#ifndef PPGPU_H_
#define PPGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define PP_OK 0
#define PP_ERR_ARG -1      /* invalid argument or parameter */
#define PP_ERR_CUDA -2     /* CUDA runtime failure (message carries the CUDA error string) */
#define PP_ERR_OVERLAP -3  /* configuration contains an overlap (main.c:57-60, MC.c:778) */
#define PP_ERR_CAPACITY -4 /* a device-side capacity was exceeded (tile particle capacity, cell grid) */
#define PP_ERR_IO -5       /* file unreadable / malformed (system.c:77-81, 245) */
#define PP_ERR_STATE -6    /* call order violated (e.g. sweeps before upload) */
#define PP_ERR_DRIFT -7    /* energy check failed: relative drift > 1e-5 (MC.c:779-781) */

/* ------------------------------------------------------------------ constants shared with the reference */
#define PP_NVT 0 /* Ensemble = 0 (defs.h:21) */
#define PP_GC 1  /* Ensemble = 1, grand canonical (defs.h:22, do_GC MC.c:31-43) */
#define PP_SUS 3 /* Ensemble = 3, successive umbrella sampling (defs.h:23, do_SUS MC.c:45-58) */
#define PP_NPT 5 /* Ensemble = 5 (defs.h:24) */

#define PP_RTMC 0  /* Dynamics = 0: roto-translations (defs.h:27) */
#define PP_VMMC 1  /* Dynamics = 1: virtual-move Monte Carlo cluster moves (defs.h:28) */
#define PP_AVBMC 2 /* Dynamics = 2: aggregation-volume-bias moves and roto-translations (defs.h:29) */

#define PP_MOVE_ROTO_TRASL 0 /* tries/accepted slots as System::tries/accepted (defs.h:11-19, 95-96) */
#define PP_MOVE_AVB 1        /* aggregation-volume-bias moves (defs.h:13) */
#define PP_MOVE_ADD 2        /* GC / SUS insertions (defs.h:14) */
#define PP_MOVE_REMOVE 3     /* GC / SUS removals (defs.h:15) */
#define PP_MOVE_VMMC 5 /* virtual-move cluster moves (defs.h:17) */
#define PP_MOVE_VOLUME 6
#define PP_MOVE_LX 7 /* the NVT box-shape move (defs.h:19) */
#define PP_N_MOVES 8

#define PP_PREC_FP32_GUARD 0 /* FP32 pair tests, FP64 re-evaluation inside the guard band (default) */
#define PP_PREC_FP64 1       /* every pair test in FP64 with the reference's operation order */

typedef struct pp_params {
	int ensemble;              /* Ensemble (system.c:62): PP_NVT or PP_NPT */
	double temperature;        /* Temperature (system.c:66) */
	double pressure;           /* P (system.c:168), NPT only */
	double disp_max;           /* Disp_max (system.c:64): translation drawn uniformly in [-Disp_max/2, Disp_max/2)^3 */
	double theta_max;          /* Theta_max (system.c:65): rotation angle uniform in [0, Theta_max) */
	double rescale_factor_max; /* rescale_factor_max (system.c:167), NPT only */
	double kf_delta;           /* KF_delta (system.c:83) */
	double kf_cosmax;          /* KF_cosmax (system.c:84) */
	uint64_t seed;             /* Seed (system.c:71): keys the counter-based Philox4x32-10 streams */
	int precision;             /* PP_PREC_FP32_GUARD or PP_PREC_FP64 */
	double guard_eps;          /* guard half-width on r^2 and on patch cosines; <= 0 selects 1e-5 */
	int resort_every;          /* checkerboard rounds between cell-grid re-sorts from the FP64 state; 0 = 4 */
	int audit;                 /* nonzero: re-check every FP32 decision in FP64 and count mismatches */
	/* Lx_move (system.c:170-196, NVT only; ignored for NPT as in the reference): once per sweep Lx changes by
	 * (R - 0.5) Lx_change_max and Ly = Lz = sqrt(V / Lx) keep the volume (MC_change_Lx, MC.c:515-585).
	 * 1 = the reference's acceptance min(1, exp(+dE / T)) (MC.c:562), 2 = the Boltzmann factor exp(-dE / T). */
	int lx_move;
	double lx_change_max;      /* Lx_change_max */
	double lyz_min, lyz_max;   /* Lyz_min, Lyz_max: allowed range of Ly = Lz (absolute lengths) */
	/* GC and SUS (system.c:90-103): Activity z; GC_N_max (GC), or Umbrella_sampling_min / _max (SUS).
	 * An engine holds one GC or SUS system; its particles are 0 .. N-1 at every moment (a removal gives the
	 * highest index to the removed particle's, as the reference does). */
	double activity;
	int n_min, n_max;
	/* Dynamics (system.c:63, MC.c:115-130): PP_RTMC, or PP_AVBMC for aggregation-volume-bias moves mixed
	 * with the roto-translations (avb.c:77-186). An AVB engine makes, per MC step, one checkerboard round of
	 * roto-translations and round((1 - avb_p) N) AVB moves, the latter one after the other on the device
	 * before each re-sort (NVT and NPT; the patches must satisfy the single-bond-per-patch condition of
	 * avb.c:14-17). */
	int dynamics;
	double avb_p; /* avb_p (avb.c:33-35): the share of roto-translations among the reference's attempts */
	/* PP_VMMC (vmmc.c:258-483): every attempt is a virtual-move cluster move, N per MC step, one after the
	 * other on the device (NVT and NPT). vmmc_max_cluster (vmmc.c:25): a cluster that reaches this size is
	 * rejected; vmmc_max_move is the reference's vmmc_max_move key, which it reads and does not use. */
	int vmmc_max_cluster;
	double vmmc_max_move;
} pp_params;

typedef struct pp_counters {
	long long tries[PP_N_MOVES];    /* System::tries (defs.h:95) */
	long long accepted[PP_N_MOVES]; /* System::accepted (defs.h:96) */
} pp_counters;

typedef struct pp_guard_stats {
	long long pairs;       /* pair tests performed by the FP32 path */
	long long fallbacks;   /* pairs inside the guard band, re-evaluated in FP64 */
	long long mismatches;  /* audit mode: FP32 decisions outside the band that FP64 contradicts (must be 0) */
	double max_err_r2;     /* audit mode: largest |r^2_fp32 - r^2_fp64| seen */
	double max_err_cos;    /* audit mode: largest |cos_fp32 - cos_fp64| seen */
	long long nl_overflows; /* neighbour lists that overflowed their capacity (those moves took the 27-cell path) */
} pp_guard_stats;

typedef struct pp_engine pp_engine;

/* Fills *p with the reference defaults this engine assumes (NVT, FP32 + guard band, eps = 1e-5). */
void pp_default_params(pp_params *p);

/* Creates an engine for one system (replaces System setup for the MC step, system_init/MC_init,
 * system.c:58-252 and MC.c:85-131). */
int pp_gpu_create(const pp_params *prm, pp_engine **out);

/* Creates an engine holding n_replicas independent systems that every sweep call advances together
 * (the batched-replica layout; no reference counterpart beyond running n copies of the reference). */
int pp_gpu_create_batch(const pp_params *prms, int n_replicas, pp_engine **out);

/* Copies one system's state to the device (the System the reference builds in system_init,
 * system.c:213-251, plus the initial energy and overlap check of main.c:55-64: returns PP_ERR_OVERLAP
 * if the configuration contains an overlap). r: N x 3, R: N x 9 row-major, box: Lx Ly Lz. A box side that
 * is not positive and finite, or a position or orientation entry that is not finite, returns PP_ERR_ARG;
 * after the latter the replica has no configuration until it is uploaded again. */
int pp_gpu_upload(pp_engine *e, int N, const double *r, const double *R, const double box[3]);
int pp_gpu_upload_replica(pp_engine *e, int replica, int N, const double *r, const double *R, const double box[3]);

/* Enqueues n MC steps (sweeps) for every replica: n calls of do_NVT (MC.c:19-29) / do_NPT (MC.c:60-68).
 * Asynchronous: returns once the work is queued; pp_gpu_sync waits for it and reports device errors. */
int pp_gpu_sweeps(pp_engine *e, long long n);
int pp_gpu_sync(pp_engine *e);

/* Tracked total energy of a replica (System::energy, updated by every accepted move, MC.c:333,501). */
int pp_gpu_get_energy(pp_engine *e, int replica, double *E);

/* Energy recomputed from scratch: 0.5 * sum_i MC_energy(i) (main.c:55-64); *overlap = 1 if any pair overlaps. */
int pp_gpu_energy(pp_engine *e, int replica, double *E, int *overlap);

/* MC_check_energy (MC.c:766-784): recompute from scratch, re-orthonormalise every orientation with
 * gram_schmidt (MC.c:774), fail with PP_ERR_OVERLAP / PP_ERR_DRIFT as the reference aborts, and
 * replace the tracked energy with the recomputed one. */
int pp_gpu_check_energy(pp_engine *e, int replica);

/* gram_schmidt on every orientation (MC.c:774, utils.c:91-113), bit-identical to the reference's. */
int pp_gpu_orthonormalise(pp_engine *e, int replica);

/* Acceptance counters (System::tries / accepted, defs.h:95-96); reset = 1 clears them afterwards as
 * output_print does (output.c:189). */
int pp_gpu_counters(pp_engine *e, int replica, pp_counters *out, int reset);

/* Copies a replica's state back: r (N x 3), R (N x 9), box, in the particle order of the upload. */
int pp_gpu_download(pp_engine *e, double *r, double *R, double box[3]);
int pp_gpu_download_replica(pp_engine *e, int replica, double *r, double *R, double box[3]);

/* Per-particle bond and overlap counts over all partners (the per-particle results of
 * output_print_bonds, output.c:213-268), in upload order. Either pointer may be NULL. */
int pp_gpu_bonds(pp_engine *e, int replica, int *n_bonds, int *n_overlaps);

/* Bonded partner lists in upload order: offsets has N+1 entries, partners capacity `cap`.
 * Returns the total number of entries (sum of n_bonds) or a negative error. If cap is short the call returns
 * PP_ERR_CAPACITY with offsets filled, so offsets[N] is the capacity needed.
 * Partners of each particle are sorted ascending (output_print_bonds lists them in cell-walk order). */
int pp_gpu_bond_lists(pp_engine *e, int replica, int *offsets, int *partners, int cap);

/* Guard-band statistics accumulated since the last call (reset = 1 clears them). */
int pp_gpu_guard_stats(pp_engine *e, pp_guard_stats *out, int reset);

/* Per-group device times collected with CUDA events on the engine's stream (pp_gpu_set_timing). */
typedef struct pp_kernel_stats {
	double sweep_ms;          /* tile sweep kernel (the checkerboard moves) */
	long long sweep_launches;
	double sort_ms;           /* grid plan + cell assignment + bin scan + scatter */
	long long sort_launches;  /* number of timed sort groups */
	double volume_ms;         /* NPT: candidate-box energy, acceptance, rescale */
	long long volume_launches;
} pp_kernel_stats;

/* Selects the CUDA device used by engines created afterwards in this thread (one process per GPU). */
int pp_gpu_select_device(int device);

/* Enables (1) or disables (0) per-group event timing of every following sweep. */
int pp_gpu_set_timing(pp_engine *e, int enable);
int pp_gpu_kernel_stats(pp_engine *e, pp_kernel_stats *out, int reset);

/* Whole re-sort periods of pp_gpu_sweeps are replayed from captured CUDA graphs (one launch per period
 * instead of one per kernel; the launches and the trajectory are the same). enable = 0 turns the graphs
 * off (every kernel launched on the stream); per-group event timing always uses stream launches. GC / SUS
 * engines and engines with AVB moves launch their kernels one by one: enable = 1 returns PP_ERR_ARG there. */
int pp_gpu_set_graphs(pp_engine *e, int enable);

/* SUS (Ensemble = 3): the histogram of N counted after every insertion / removal attempt (MC.c:50), bins
 * Umbrella_sampling_min .. Umbrella_sampling_max, into hist (may be NULL); reset = 1 clears it, as
 * output_and_reset_sus does at every print (output.c:343-356, main.c:89). Insertions and removals
 * (MC_add_remove, MC.c:342-448) run once per re-sort period, N_max x 0.01 attempts per MC step as the
 * reference makes on average, one after the other with exact FP64 energies. */
int pp_gpu_sus_histogram(pp_engine *e, long long *hist, int reset);

/* Plain rounds over the neighbour lists as one persistent cooperative kernel (enable = 1): the 8 colours
 * of a round (the 8 sublattice passes of do_NVT/do_NPT's sweep, MC.c:19-29, 60-68) in one launch, with
 * a grid barrier between colours. enable = 0 (the default) launches one kernel per colour. The
 * trajectory is the same bit for bit either way. */
int pp_gpu_set_persistent(pp_engine *e, int enable);

/* Failure-detection hook of that kernel's grid barrier (no counterpart in the reference). limit_cycles:
 * SM clock cycles a barrier wait may spin before it gives up (0 = the default, about one second).
 * unreachable = 1 makes the first barrier of every round wait for one arrival more than the grid makes,
 * so every wait runs out: the kernel returns early and the next call that reads the engine's state
 * (counters, energy, download) returns PP_ERR_CUDA, "grid barrier wait timed out". The engine's state is
 * then incomplete; destroy it. The GPU stays usable: no wait is unbounded. */
int pp_gpu_set_barrier_test(pp_engine *e, long long limit_cycles, int unreachable);

/* Per-epoch neighbour lists (default on). Between two re-sorts no particle leaves its cell and each moves
 * at most once per round, so after every re-sort each particle's candidates in the 27 surrounding cells
 * that lie closer than a radius covering the epoch's largest possible motion (and, for NPT, its accepted
 * compressions) are listed, and plain moves test only those pairs. A pair left out can neither overlap nor
 * bond during the epoch, so the decisions, hence the trajectory, are the full 27-cell scan's bit for bit.
 * enable = 0 scans the 27 cells in every move. No counterpart in the reference, whose MC_energy walks the
 * 27 cell lists on every call (MC.c:272-309). */
int pp_gpu_set_neighbour_lists(pp_engine *e, int enable);

/* Enqueues n sweeps between two CUDA events recorded on the engine's stream, waits, and returns the
 * elapsed device time in *ms. */
int pp_gpu_time_sweeps(pp_engine *e, long long n, double *ms);

/* Allocation-free energy of one configuration (no counterpart in the reference: an addition for callers
 * that may not allocate device memory themselves -- hosts that run the engine inside a device-memory
 * budget or pool owned by someone else, and latency-sensitive loops, where cudaMalloc/cudaFree could
 * fail or stall the whole device with their implicit synchronisation).
 *
 * The caller passes device pointers: r_dev (N x 3 doubles) and R_dev (N x 9 doubles, orientation rows),
 * and optionally n_bonds_dev / n_overlaps_dev (N ints each, may be NULL), which receive the per-particle
 * bond and overlap counts in input order, as pp_gpu_bonds does. *E receives 0.5 * sum_i MC_energy(i)
 * (main.c:55-64 semantics; -bonds) and *overlap whether any pair overlaps. Model: KF_delta, KF_cosmax,
 * FP32 pair tests with the FP64 guard band (eps = 1e-5), bit-identical decisions to the reference.
 *
 * Nothing is allocated by the call: all scratch (cell grid, sort buffers, working records) lives in one
 * static device array of about 11.2 MiB. The array comes into existence when the library's kernel module
 * is loaded on a device -- under CUDA's lazy module loading (the default) that is the first engine or
 * pp_gpu_energy_noalloc call on that device -- and stays until the process exits. A caller on a tight
 * device-memory budget should therefore make one call at start-up, outside that budget; a failure to
 * load the module there is reported as PP_ERR_CUDA "cudaGetSymbolAddress".
 * Limits: N <= 32768 particles and at most 131072 cells (even cell count >= 4 per axis, cell edge >=
 * 1 + KF_delta, i.e. roughly a 57^3 box at delta = 0.12); larger inputs return PP_ERR_CAPACITY with a
 * message in err (err may be NULL). N = 0 is valid (E = 0, no overlap).
 * Every call looks up the array's device address with cudaGetSymbolAddress, with the calling thread's
 * current device and context, so a device reset between calls is harmless.
 * Streams: a call copies with cudaMemcpy/cudaMemset and launches on the legacy default stream, and
 * returns after the result is on the host. No call may be made while any stream of the process is being
 * captured. Inputs written on a non-blocking stream (cudaStreamNonBlocking, e.g. a framework's pooled
 * side streams) are not ordered before the call's reads: synchronise those producers first. Calls share
 * the array, which keeps the last call's contents (each call writes everything it reads): calls that
 * overlap on the GPU (from several host threads) race on it and must be serialised by the caller.
 * Returns PP_OK, PP_ERR_ARG, PP_ERR_CAPACITY or PP_ERR_CUDA. */
int pp_gpu_energy_noalloc(int N, const double *r_dev, const double *R_dev, const double box[3], double kf_delta, double kf_cosmax,
		int *n_bonds_dev, int *n_overlaps_dev, double *E, int *overlap, char *err, int err_len);

/* ------------------------------------------------------------------ learned proposal: the network */
/* Per-particle MLP 36 -> 64 -> 64 -> 4 (ReLU), BF16 operands on the tensor cores, FP32 accumulation.
 * No counterpart in the reference: an addition to it, whose plain fallback is MC_move_rototranslate.
 * Parameters are FP32, laid out W1[64][36] b1[64] W2[64][64] b2[64] W3[4][64] b3[4] (PP_MLP_NPARAMS). */
#define PP_MLP_IN 36
#define PP_MLP_HIDDEN 64
#define PP_MLP_OUT 4
#define PP_MLP_NPARAMS 6788
#define PP_MLP_SAMPLE 40 /* floats per training sample: 36 features + 4 component utilities */

/* z[n][4] = network(x[n][36]) on the current device (host arrays; allocates device scratch). */
int pp_mlp_forward(const float *params, int n, const float *x, float *z);

/* Gradient of L = -(1/n) sum_s J_s over n training samples (samples[n][40]: features, utilities u_k),
 * J = sum_k pi_k u_k + tau H(softmax z), pi = (1 - floor) softmax(z) + floor e_0, into grad[PP_MLP_NPARAMS]
 * (same layout as params); *objective (may be NULL) receives the mean J. tiles_per_cta: 128-sample tiles
 * each CTA accumulates in tensor memory before its atomics (the engine's training uses the same kernel). */
int pp_mlp_grad(const float *params, int n, const float *samples, double floor, double tau, int tiles_per_cta, float *grad, double *objective);

/* Failure-detection hook of the tensor-core waits (no counterpart in the reference). The network's kernels
 * wait for each batch of tcgen05 MMAs on an mbarrier, at most about one second of SM clock cycles; a wait
 * that runs out sets a sticky error, the kernel stops issuing tensor-core work and returns, and the entry
 * point returns PP_ERR_CUDA. This runs that same bounded wait in one warp on a barrier of its own, with
 * limit_cycles (1 .. the one-second default) as its limit: arrive = 1 arrives first, so the wait completes;
 * arrive = 0 arrives never (and issues no tensor-core work), so the wait runs out. *timed_out and *cycles
 * (either may be NULL) receive whether it gave up and how long it waited. Returns PP_OK, PP_ERR_CUDA when
 * the wait ran out (the context stays usable), or PP_ERR_ARG. */
int pp_mlp_wait_test(long long limit_cycles, int arrive, int *timed_out, long long *cycles);

/* ------------------------------------------------------------------ learned proposal: the engine */
/* With the learned proposal on, every attempt of pp_gpu_sweeps draws its move from a four-component
 * mixture: component k displaces uniformly in a cube of edge scale_disp[k] * Disp_max and rotates by an
 * angle uniform below scale_theta[k] * Theta_max (capped below pi) about a uniform axis; component 0 is
 * the plain move (scales 1). The weights are pi = (1 - floor) softmax(network(features)) + floor e_0,
 * where the features are up to 12 neighbour patch sites (3 nearest neighbours within 1 + KF_delta, 4
 * patches each, centre + 0.5 patch direction) in the particle's frame, zero-padded. Acceptance is
 * Metropolis-Hastings with the reverse-move density, so the Boltzmann distribution is kept exactly.
 * The network is trained on the GPU (pp_gpu_learned_train) on samples of configurations generated by
 * the plain move (pp_gpu_learned_collect); per sample and component the utility is the mean over
 * `draws` proposals of kappa |bond change| min(1, exp(-(dE - 1) / T)) + jump acc (|d|^2 / Disp_max^2 +
 * angle^2 / Theta_max^2), acc = min(1, exp(-dE / T)) (0 for an overlap or a move out of the cell): how
 * often the component proposes a change of the particle's bond count that is no less likely to be
 * accepted than breaking one bond, with the squared jump as a tie-break; divided by the sample's largest
 * utility (so every environment's preference counts alike). */
#define PP_PROPOSAL_PLAIN 0
#define PP_PROPOSAL_LEARNED 1
#define PP_MIX 4

typedef struct pp_learned_params {
	double scale_disp[PP_MIX];  /* cube edge of component k in units of Disp_max (scale_disp[0] = 1) */
	double scale_theta[PP_MIX]; /* maximum angle of component k in units of Theta_max (scale_theta[0] = 1) */
	double floor;               /* weight of the plain component always mixed in, (0, 1] */
	double entropy;             /* training: entropy bonus tau of the objective (>= 0) */
	double kappa;               /* training: weight of the bond-count change in the utility (>= 0) */
	double jump;                /* training: weight of the squared jump in the utility (>= 0; a tie-break) */
	int draws;                  /* training: proposals per component and sample, [1, 64] */
	uint64_t seed;              /* initial weights and the training order */
} pp_learned_params;

void pp_default_learned_params(pp_learned_params *p);

/* Allocates the network (seeded initial weights: uniform fan-in hidden layers, zero output layer, i.e.
 * the uniform mixture) and the training state; may be called again to reset. */
int pp_gpu_learned_init(pp_engine *e, const pp_learned_params *p);
int pp_gpu_learned_set_weights(pp_engine *e, const float *params); /* PP_MLP_NPARAMS floats */
int pp_gpu_learned_get_weights(pp_engine *e, float *params);

/* PP_PROPOSAL_PLAIN (default) or PP_PROPOSAL_LEARNED (needs pp_gpu_learned_init) for the following sweeps. */
int pp_gpu_set_proposal(pp_engine *e, int proposal);

/* n_configs times: sweeps_between sweeps with the plain move, then samples_per_config training samples of
 * the current configuration appended to the engine's sample buffer (one checkerboard colour's attempts,
 * spread over its list). */
int pp_gpu_learned_collect(pp_engine *e, int n_configs, int sweeps_between, int samples_per_config);

/* epochs passes over the sample buffer in shuffled 128-sample tiles, one Adam step (learning rate lr)
 * per batch of tiles_per_cta x (SMs) tiles; *objective (may be NULL) = mean J over the last epoch. */
int pp_gpu_learned_train(pp_engine *e, int epochs, int tiles_per_cta, double lr, double *objective);

/* Number of samples in the buffer; if out is not NULL, copies them (count x PP_MLP_SAMPLE floats). */
int pp_gpu_learned_samples(pp_engine *e, long long *count, float *out);
int pp_gpu_learned_clear_samples(pp_engine *e);

/* The 36 features of every particle of a replica in the current state (N x 36, particle order). */
int pp_gpu_learned_features(pp_engine *e, int replica, float *features);

/* Attempts and acceptances of learned moves per mixture component since the last reset (all replicas). */
int pp_gpu_learned_stats(pp_engine *e, long long tries[PP_MIX], long long accepted[PP_MIX], int reset);

/* ------------------------------------------------------------------ autotuner */
/* Chooses the engine's schedule on the live system by timing it: the checkerboard rounds between cell-grid
 * re-sorts (1, 2, 4, 8, 16), the re-sorts between physical reorders of the FP64 state (4, 16, 64), the cell
 * edge as a multiple of its minimum (1.0, 1.2, 1.5: the cell occupancy, hence attempts per round and
 * neighbours per attempt) and, when they are enabled, the neighbour lists on or off (their radius grows
 * with the re-sort period). Each candidate runs 2 + trial_sweeps ordinary sweeps (they are part of the
 * trajectory) timed with CUDA events; the one with the most move attempts per second is kept. NPT replicas
 * keep the compression margin of their cell edge for every candidate period. No counterpart in the
 * reference. */
typedef struct pp_tune_result {
	int resort_every;                /* chosen */
	int reorder_every;               /* chosen */
	double cell_scale;               /* chosen */
	double attempts_per_s;           /* of the chosen schedule */
	double baseline_attempts_per_s;  /* of the schedule before tuning */
	int n_tried;
	int neighbour_lists;             /* chosen (tried both ways when the lists are enabled) */
} pp_tune_result;

int pp_gpu_autotune(pp_engine *e, int trial_sweeps, pp_tune_result *out);

/* Number of replicas, particles of a replica, current box of a replica. */
int pp_gpu_num_replicas(const pp_engine *e);
int pp_gpu_num_particles(const pp_engine *e, int replica);
int pp_gpu_box(pp_engine *e, int replica, double box[3]);

/* Number of kernel launches the engine has enqueued since creation (its own kernels only). */
long long pp_gpu_launch_count(const pp_engine *e);

const char *pp_gpu_last_error(const pp_engine *e);
void pp_gpu_destroy(pp_engine *e);

/* ------------------------------------------------------------------ reference file formats (host only) */
/* .rrr header "step N Lx Ly Lz" (system.c:80; output.c:306). Returns PP_OK or PP_ERR_IO. */
int pp_rrr_header(const char *path, long long *step, int *N, double box[3]);

/* Reads a .rrr configuration exactly as system_init does (system.c:213-243): each particle's two stored
 * orientation rows are normalised, the third row is their cross product and the matrix is passed through
 * gram_schmidt, so R is bit-identical to the reference's. r: N x 3, R: N x 9. Returns PP_OK, PP_ERR_IO
 * (unreadable or malformed file, a particle count other than N; message in err) or PP_ERR_ARG. */
int pp_rrr_read(const char *path, int N, double *r, double *R, double box[3], char *err, int err_len);

/* Writes a .rrr configuration in output_save's format (output.c:302-317). Returns PP_OK, PP_ERR_ARG, or
 * PP_ERR_IO when the file cannot be opened or a write fails (e.g. a full disk). */
int pp_rrr_write(const char *path, long long step, int N, const double *r, const double *R, const double box[3]);

/* Seeded random sequential insertion of N non-overlapping unit spheres at the given density in a cubic box,
 * with uniformly random orientations: the algorithm of the reference generator (generator.c:43-68,
 * 86-124; random_orientation, utils.c:133-169), drawing from the drand48 recurrence seeded as
 * srand48(seed). Returns PP_ERR_ARG for density > 0.7 (generator.c:99-102). If round_like_file is
 * nonzero, orientations pass through the same "%lf" text rounding and re-orthonormalisation that writing
 * and reading a .rrr file applies, so the result equals loading the generator's file. */
int pp_generate(int N, double density, int seed, int round_like_file, double *r, double *R, double box[3]);

#ifdef __cplusplus
}
#endif

#endif /* PPGPU_H_ */
