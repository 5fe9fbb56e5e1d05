/*
 * ppgpu_internal.h -- data layout shared by the C host code (ppgpu_host.c) and the CUDA kernels
 * (ppgpu_kernels.cu). Plain C structs; no torch types.
 *
 * Device memory (one engine = R replicas; particle "slots" are global over replicas):
 *   rec[slot]   16 doubles, the canonical FP64 state:
 *                 [0..2]  x y z (unwrapped position)
 *                 [3..6]  q = (w, x, y, z), accumulated rotation quaternion (not normalised)
 *                 [7..15] R0, orientation rows at upload (or at the last orthonormalisation)
 *               The orientation is R = R0 . Q(q) with Q the rotation matrix of q / |q| (orient64), so an
 *               accepted rotation costs one FP64 quaternion product instead of a 3x3 matrix product, and
 *               an uploaded orientation is reproduced bit for bit while q is the identity.
 *               Only FP64 arithmetic ever writes it.
 *   spos[k]     float4 (lx, ly, lz, slot) of the particle at cell-sorted position k, cell-local, 0 <= l < w
 *   sori[3k..]  3 x float4 orientation columns c_j = (R0j, R1j, R2j) of the same particle:
 *                 (c0x, c0y, c0z, c1x) (c1y, c1z, c2x, c2y) (c2z, id, cell, -)
 *               id = particle index in its replica, cell = global cell index.
 *               spos/sori are rebuilt from rec every `resort_every` rounds and updated in FP32 by accepted
 *               moves in between; the distance filter reads only spos (16 B per candidate).
 *   cell_start  per replica n_x*n_y*n_z + 1 entries (global cell index = replica cell base + local index,
 *               local index = (cz * n_y + cy) * n_x + cx), particles of a cell contiguous in spos/sori.
 *   clist       per colour (8), the non-empty cells of that checkerboard colour as int4 (global cell,
 *               first sorted position, particle count, replica).
 */
#ifndef PPGPU_INTERNAL_H_
#define PPGPU_INTERNAL_H_

#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPI_REC 16
#define PPI_Q 3   /* offset of q in rec */
#define PPI_R0 7  /* offset of R0 in rec */
#define PPI_MAX_AXIS_CELLS 1024

/* error codes written by kernels into ppi_rstate.error */
#define PPI_E_GRID 2  /* the box became too small for an even cell grid of edge >= r_cut */
#define PPI_E_EXACT 3 /* more undecidable pairs in one warp's share of a volume pass than it keeps */
#define PPI_E_LISTS 4 /* more guard-band pairs in one volume pass than its buffer holds */
#define PPI_E_BARRIER 5 /* a grid-barrier wait of the persistent round kernel ran out of its limit */
#define PPI_E_GCFULL 6  /* a grand-canonical insertion found the system at GC_N_max (the reference stops there) */
#define PPI_E_AVB 7     /* an AVB move's rejection sampling ran out of its draw limit (no move made) */
#define PPI_E_VMMC 8    /* a VMMC move ran out of link memory or moved a cluster into an overlap (the reference stops) */

typedef struct ppi_rparams {
	int N;           /* particles of this replica */
	int p0;          /* first slot */
	int ensemble;    /* 0 NVT, 1 GC, 3 SUS, 5 NPT */
	int precision;   /* 0 FP32 + guard, 1 FP64 */
	int audit;
	int cell_base;   /* first global cell index of this replica */
	int cell_cap;    /* cells reserved for this replica */
	int lx_move;     /* NVT box-shape move (MC.c:515-585): 0 off, 1 reference acceptance, 2 Boltzmann acceptance */
	double T, P, disp_max, theta_max, rescale_max;
	double cosmax, sqr_rcut, r_cut, w_min;
	double base[4][3];     /* tetrahedral base patches, bit-identical to system.c:20-31 */
	uint64_t acc_thr[32];  /* accept a move with dE = +k iff U53 < acc_thr[k], U53 uniform in [0, 2^53) */
	float cosmax_f, sqr_rcut_f, eps_f, disp_max_f, theta_max_f, base_f;
	float nl_r2f;          /* squared radius of the per-epoch neighbour lists (0: no lists, exact path) */
	float pad1;
	uint64_t seed;
	double lx_change_max, lyz_min, lyz_max; /* Lx_change_max, Lyz_min, Lyz_max (system.c:177-179) */
	double activity;       /* GC / SUS: Activity z (system.c:91) */
	int n_min, n_max;      /* GC / SUS: the particle-number window (GC: 0 and GC_N_max) */
	/* Dynamics = 2 (avb.c): aggregation-volume-bias moves between the checkerboard rounds */
	int dynamics;          /* 0 roto-translations only, 2 roto-translations and AVB moves */
	int avb_head0;         /* first entry of this replica's AVB cell heads */
	int avb_ncap[3];       /* cells per axis the heads were reserved for */
	int avb_per_step;      /* AVB attempts per MC step: round((1 - avb_p) N) */
	double avb_vin, avb_vout; /* AVBMC_init's bonding and non-bonding volumes (avb.c:26-28), fixed at upload */
	double base_orient[9]; /* a rotation taking base patch 0 to (0, 0, 1) (system.c:33-54) */
	int vmmc_max_cluster;  /* Dynamics = 1 (vmmc.c): a cluster that reaches this size is rejected */
	int pad_vmmc;
} ppi_rparams;

typedef struct ppi_rstate {
	double box[3];
	double V;                    /* System::V (updated by accepted volume moves, MC.c:500) */
	long long bonds;             /* tracked bonded pairs: energy = -bonds */
	unsigned long long tries[8];
	unsigned long long accepted[8];
	long long vol_bonds;         /* bonds counted by the last energy pass (candidate box for NPT) */
	int vol_overlap;
	int vol_accept;
	int error;
	int error_info;
	unsigned long long pairs, fallbacks, mismatches;
	unsigned int max_err_r2_bits, max_err_cos_bits;
	unsigned long long nl_overflow; /* particles whose neighbour list overflowed (their attempts take the exact path) */
	int n_live;                  /* GC / SUS: current particle count (slots p0 .. p0 + n_live - 1 hold them) */
	int pad_live;
} ppi_rstate;

typedef struct ppi_grid {
	int n[3];          /* cells per axis (even) */
	int ncells;
	double w[3];       /* cell edge */
	double shift[3];   /* grid origin offset, uniform in [0, w) at every re-sort */
	double inv_w[3], inv_L[3];
	float wf[3];
	float pad;
	float inv_wf[3], inv_Lf[3], Lf[3]; /* FP32 copies for the cell assignment's guesses */
	float pad4;
	float shiftf[3];   /* FP32 copy of shift (the cell assignment's guesses) */
	float pad5;
	/* candidate box of the current sweep's NPT volume move (MC.c:456-472) or Lx move (MC.c:520-537) */
	int vol_dir;       /* NPT: the scaled axis; PPI_LX_DIR: Lx move; -1: no candidate */
	int vol_mask;      /* bit k: axis k is scaled in the candidate box */
	double vol_f, vol_V1, vol_V0; /* NPT: scale factor of axis vol_dir, volumes before and after */
	double vol_f3[3];  /* per-axis scale factors of the candidate (1 on unscaled axes) */
	double vol_box3[3]; /* candidate box sides */
	float vol_ff3[3];  /* FP32 copies of vol_f3 */
	float pad3;
} ppi_grid;
#define PPI_LX_DIR 3

/* learned proposal: the four mixture components (component 0 is the plain move) and training knobs */
#define PPI_MIX 4
typedef struct ppi_learn {
	float sdisp[PPI_MIX];  /* component k draws its displacement in a cube of edge sdisp[k] * Disp_max */
	float stheta[PPI_MIX]; /* ... and its rotation angle uniformly below stheta[k] * Theta_max (capped below pi) */
	float floor0;          /* weight of the plain component added to the network's softmax */
	float kappa;           /* training utility: weight of the accepted bond-count change */
	float jump;            /* training utility: weight of the accepted squared jump (tie-break) */
	int draws;             /* training utility: proposals per component and sample */
} ppi_learn;

/* per replica, the learned mixture in that replica's units (host-computed, the kernels' own FP32 values) */
#define PPI_LEXP 8
typedef struct ppi_lrep {
	double v[PPI_MIX];           /* 1 / (a_k^3 t_k): density of component k inside its support */
	double expk[2 * PPI_LEXP + 1]; /* exp(-k / T), k = -8..8 */
	float a[PPI_MIX];            /* cube edge of component k: Disp_max * sdisp[k] (FP32) */
	float t[PPI_MIX];            /* maximum angle: min(Theta_max * stheta[k], largest FP32 below pi) */
} ppi_lrep;

/* device counters of the captured sweep graphs: a kernel given a negative round / epoch / sweep argument
 * (-1 - k) uses the k-th index after these (the host writes them before each replay) */
typedef struct ppi_ctr {
	long long round, epoch, sweep;
	int vol_any; /* some replica accepted the current volume move (k_vol_apply has work) */
	int pad;
} ppi_ctr;

/* all device pointers, passed by value to every kernel */
typedef struct ppi_dev {
	int nrep;
	int ntot;          /* total slots */
	int total_cells;   /* sum of cell caps */
	int pad;
	double *rec;
	float4 *spos;      /* 1 x float4 per particle */
	float4 *sori;      /* 3 x float4 per particle */
	int *id;           /* slot -> particle index in its replica */
	int *rep;          /* slot -> replica */
	int *cellof;       /* slot -> global cell (current grid) */
	int *cell_count;
	int *cell_start;   /* total_cells + 1 */
	int *cell_part;    /* k_scan's tile-local exclusive prefix of cell_count */
	int *cell_rep;     /* global cell -> replica */
	int *scan_aux;
	int4 *clist;       /* 8 lists of capacity clist_cap each */
	int *ccount;       /* 8 colour-list counters, [8]: k_scan's ticket */
	unsigned char *dflag; /* 8 x clist_cap: deferred attempts a warp could not keep in shared memory */
	unsigned char *eflag; /* ntot: the same for particles of the energy pass */
	int audit_any;     /* some replica audits: every pass runs in audit mode */
	int lanes;         /* lanes per attempt of the colour and energy passes (4 or 8; 0 = default) */
	int clist_cap;
	int nl_k;          /* neighbour-list capacity per particle (multiple of 4; 0 = no lists) */
	ppi_rparams *rp;
	ppi_rstate *rs;
	ppi_grid *grid;
	int *out_bonds;    /* per slot */
	int *out_overlaps;
	int *out_partners; /* bond lists: per slot up to PPI_MAX_PARTNERS */
	double *tmp_rec;   /* reorder / export scratch (ntot records) */
	int *tmp_id;
	/* learned proposal (allocated when it is first configured) */
	float4 *simg;                 /* per sorted position, 4 x float4: FP32 image of the canonical state (position
	                                 wrapped into the box, particle id, orientation rows), a function of rec, id
	                                 and the box only */
	const struct ppi_lrep *lrep;  /* per replica: the mixture components' edges, angles, densities */
	const unsigned char *mlp_img; /* packed BF16 network operands (ppgpu_umma.cuh) */
	const ppi_learn *learn;
	float *samples;               /* training samples [sample_cap][40] */
	float *feat;                  /* per slot features [ntot][36] (pp_gpu_learned_features) */
	unsigned long long *lstats;   /* per component: tries [0..3], accepted [4..7] */
	int *lerr;                    /* tensor-core barrier timeouts of the learned passes */
	int sample_cap;
	int pad2;
	ppi_ctr *ctr;                 /* graph-path counters */
	/* per-epoch neighbour lists, per sorted position: nl[k * nl_k + j] = candidate sorted position << 5 |
	 * cell offset code (dx + 1) + 3 (dy + 1) + 9 (dz + 1); nl_cnt[k] = entries (> nl_k: overflow) */
	int *nl;
	int *nl_cnt;
	/* the epoch's pairs for the volume pass, each once: (lower sorted position i, candidate << 5 | code) */
	int2 *vpairs;
	int *vp_count;     /* [0] pairs written by the list build, [1] particles in vp_over */
	int *vp_over;      /* sorted positions whose list overflowed: their half shell is scanned in the cells */
	int *srep;         /* replica of each sorted position */
	int vp_cap;
	int vun_cap;
	int2 *vunsure;     /* guard-band pairs of the current volume pass, decided in FP64 after it */
	int *vun_count;
	/* the persistent round kernel (k_round): the 8 colours of a round in one cooperative launch, a grid
	 * barrier between colours. gbar[0] = CTA arrivals, gbar[1 + c] = the work counter of the round's c-th
	 * colour (both cleared before each launch), gbar[15] = sticky error: a barrier wait that ran out of its
	 * limit (PPI_E_BARRIER) */
	int *gbar;
	long long bar_limit; /* SM clock cycles a barrier wait may spin before it gives up (0: default ~1 s) */
	int bar_extra;       /* test hook: arrivals the first barrier waits for beyond the grid (1 = never completes) */
	int persist;         /* 1: plain rounds over the neighbour lists use k_round, 0: one launch per colour */
	unsigned long long *sus_hist; /* SUS: histogram of N after every insertion/removal attempt, n_max - n_min + 1 bins */
	/* AVB and VMMC moves: linked cells (cells.c) of the replica's live particles, rebuilt at every batch */
	int *avb_head;     /* per replica avb_ncap[0] x [1] x [2] entries from avb_head0: first slot offset, -1 */
	int *avb_next;     /* per slot: next slot offset of its cell, -1 */
	int *avb_cell;     /* per slot: its cell */
	/* VMMC (vmmc.h: vmmc_d), per slot: the stored degrees of freedom (x y z and 9 orientation entries),
	 * the possible links (16 pairs of slot offsets per slot of the replica), the prelinked and outright
	 * failed lists (16 entries per slot each), link counters, copies, cluster flags and the cluster */
	double *vm_old;
	int *vm_links, *vm_pre, *vm_fail;
	int *vm_cnt, *vm_copies, *vm_in, *vm_clust;
} ppi_dev;

#define PPI_MAX_PARTNERS 24

/* launchers (ppgpu_kernels.cu); each returns a cudaError_t value as int and adds its launches to *nl */
int ppi_resort(const ppi_dev *d, long long epoch, cudaStream_t s, long long *nl);
/* use_nl: the epoch's neighbour lists are valid (built by ppi_nlist after the re-sort, plain moves since) */
int ppi_round(const ppi_dev *d, long long round, const int *colours, int audit, int use_nl, cudaStream_t s, long long *nl);
/* neighbour lists of every sorted position for the current epoch (after ppi_resort) */
int ppi_nlist(const ppi_dev *d, cudaStream_t s, long long *nl);
int ppi_energy(const ppi_dev *d, int mode, cudaStream_t s, long long *nl);
/* use_nl: the candidate-box energy takes its pairs from the epoch's neighbour lists (every replica has them) */
int ppi_volume(const ppi_dev *d, long long sweep, int use_nl, cudaStream_t s, long long *nl);
int ppi_gram_schmidt(const ppi_dev *d, int first, int count, cudaStream_t s, long long *nl);
/* GC / SUS: `attempts` sequential insertion / removal attempts per replica (MC_add_remove, MC.c:342-448) */
int ppi_exchange(const ppi_dev *d, long long step, int attempts, cudaStream_t s, long long *nl);
/* Dynamics = 2: `steps` MC steps' worth of AVB attempts per AVB replica (AVBMC_dynamics, avb.c:77-186) */
int ppi_avb(const ppi_dev *d, long long step, int steps, cudaStream_t s, long long *nl);
/* Dynamics = 1: `steps` MC steps of VMMC moves (N each) per VMMC replica (VMMC_dynamics, vmmc.c:258-483) */
int ppi_vmmc(const ppi_dev *d, long long step, int steps, cudaStream_t s, long long *nl);
int ppi_reorder(const ppi_dev *d, cudaStream_t s, long long *nl);
/* writes x y z R00..R22 (12 doubles) of slots [first, first + count) into d->tmp_rec */
int ppi_export(const ppi_dev *d, int first, int count, cudaStream_t s, long long *nl);
int ppi_sm_count(void);
/* sizes the launch grids of every pass once (their occupancy queries must not run inside a stream capture) */
int ppi_prepare(const ppi_dev *d);
/* writes the graph-path counters (one small kernel on the stream) */
int ppi_set_counters(const ppi_dev *d, long long round, long long epoch, long long sweep, cudaStream_t s, long long *nl);

/* learned proposal (ppgpu_kernels.cu): canonical images of all slots; one round of learned moves; the
 * features of every slot; training samples of the current state for colour col into rows [base, base + count) */
int ppi_canon(const ppi_dev *d, cudaStream_t s, long long *nl);
int ppi_round_learned(const ppi_dev *d, long long round, const int *colours, int audit, cudaStream_t s, long long *nl);
int ppi_learn_features(const ppi_dev *d, cudaStream_t s, long long *nl);
int ppi_learn_collect(const ppi_dev *d, long long snap, int col, int base, int count, cudaStream_t s, long long *nl);
/* the network (ppgpu_mlp.cu) */
int ppi_mlp_pack(const float *P_dev, unsigned char *img_dev, cudaStream_t s);
int ppi_mlp_train_step(const unsigned char *img, const float *samples, int n_samples, const int *tile_ids, int n_tiles, int tiles_per_cta, float floor0,
		float tau, float inv_batch, float *grad, double *objective, int *err_dev, cudaStream_t s);
int ppi_mlp_adam(float *P, float *grad, float *m1, float *m2, unsigned char *img, int step, float lr, cudaStream_t s);

/* model parameters of one NVT system of N particles (exact FP64 base patches, FP32 thresholds),
 * without cell capacities; defined in ppgpu_host.c (compiled with -ffp-contract=off) */
void ppi_model_params(int N, double kf_delta, double kf_cosmax, ppi_rparams *rp);

/* energy kernel modes */
#define PPI_EN_BONDS 0    /* per-slot bond/overlap counts + per-replica sum into rs.vol_bonds */
#define PPI_EN_VOLUME 1   /* NPT candidate box: per-replica sums only */
#define PPI_EN_PARTNERS 2 /* as BONDS, and bonded partner ids per slot into out_partners */

#ifdef __cplusplus
}
#endif

#endif /* PPGPU_INTERNAL_H_ */
