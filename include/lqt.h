/*
 * lqt.h -- C ABI of the GB300 monodomain TPORd simulator.
 *
 * This is the drop-in boundary for the reference's hot path.  The reference
 * (ShugangZhang/LQT1) exposes no library: its boundary is the `Cell` virtual
 * interface implemented by `TPORd` (SingleCell/Cell.cc:22-42,
 * SingleCell/TPORd.cc:137-376) and the CUDA kernels `calc_du`, `init_Istim`,
 * `set_Istim`, `set_S2Istim`, `Itot`, `new_u_v` driven by the host loops in
 * GPU3D.cu:1731-1842 and new_11.cu:1755-1890.  Each entry point below names the
 * reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an lqt status code; none exits, prints or blocks
 *    on input (the reference's HandleError waits on `cin`, GPU3D.cu:111-118).
 *  - Pointers named *_host are host memory; *_dev are device memory on the
 *    handle's device.  Sizes are element counts.
 *  - State vectors use the reference text-dump order (LQT_S_* below,
 *    SingleCell/TPORd.cc:200-252), 40 doubles per cell.
 *  - A handle is not thread-safe; distinct handles may be used concurrently.
 */
#ifndef LQT_H_
#define LQT_H_

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    LQT_OK = 0,
    LQT_ERR_INVALID = 1,        /* bad argument or size */
    LQT_ERR_CUDA = 2,           /* a CUDA runtime call failed */
    LQT_ERR_NUMERIC = 3,        /* blow-up detector tripped (NaN or V outside range) */
    LQT_ERR_TIMEOUT = 4,        /* a bounded device wait gave up */
    LQT_ERR_NOMEM = 5,          /* device or host allocation failed */
    LQT_ERR_STATE = 6,          /* call out of order (e.g. results before a run) */
    LQT_ERR_IO = 7              /* file open/read/write failed */
};

/* ---- cell types: the reference CPU enum (SingleCell/Cell.cc:20) --------- */
enum {
    LQT_LVEPI = 0,
    LQT_LVENDO = 1,
    LQT_EPI = 2,
    LQT_ENDO = 3,
    LQT_MCELL = 4,
    LQT_EMPTY = 255             /* grid voxel that is not tissue */
};

/* ---- precision forms --------------------------------------------------- */
enum {
    LQT_FP64 = 0,               /* plain FP64 everywhere (the reference's arithmetic) */
    LQT_MIXED = 1               /* FP32 gates/currents/diffusion, FP64 concentrations */
};

/* ---- state order (SingleCell/TPORd.cc:200-252) ------------------------- */
enum {
    LQT_S_V = 0, LQT_S_NAI, LQT_S_NASS, LQT_S_KI, LQT_S_KSS, LQT_S_CAI,
    LQT_S_CASS, LQT_S_CANSR, LQT_S_CAJSR, LQT_S_SM, LQT_S_SH, LQT_S_SJ,
    LQT_S_HSP, LQT_S_JP, LQT_S_ML, LQT_S_HL, LQT_S_HLP, LQT_S_A, LQT_S_IF,
    LQT_S_IS, LQT_S_AP, LQT_S_IFP, LQT_S_ISP, LQT_S_D, LQT_S_FF, LQT_S_FS,
    LQT_S_FCAF, LQT_S_FCAS, LQT_S_JCA, LQT_S_NCA, LQT_S_FFP, LQT_S_FCAFP,
    LQT_S_XRF, LQT_S_XRS, LQT_S_XS1, LQT_S_XS2, LQT_S_XK1, LQT_S_JRELNP,
    LQT_S_JRELP, LQT_S_CAMKT,
    LQT_NSTATE = 40
};

/*
 * Scenario parameters: the runtime form of the reference's compile-time
 * scenario macros (BASELINE/CON/LQT1/ISO1/SUPREP, SingleCell/TPORd.cc:30-36,
 * GPU3D.cu:18-22, new_11.cu:18-21).  A factor of exactly 1 (or shift 0)
 * leaves the arithmetic bit-identical to the build without the macro.
 */
typedef struct lqt_model {
    double dss_shift;      /* ISO1 d-gate shift, mV: 12 (TPORd.cc:582); 0 = off */
    double fss_shift;      /* ISO1 f-gate shift, mV: 8 (TPORd.cc:588); 0 = off */
    double pca_scale;      /* ISO1 PCa factor: 1.6 CPU (TPORd.cc:629), 3.5 2D
                              (new_11.cu:812), 4 3D (GPU3D.cu:767); 1 = off */
    double gks_scale;      /* LQT1 GKs factor: 0.05 (TPORd.cc:705-707); 1 = off */
    double gks_iso_scale;  /* ISO1 GKs factor: 3.2 (TPORd.cc:731-733); 1 = off */
    double suprep_dose;    /* SUPREP dose in fmol (TPORd.cc:709-728); <= 0 = off */
    double reserved[2];    /* must be zero */
} lqt_model;

/* Presets reproducing the reference's builds. */
enum {
    LQT_PRESET_BASELINE = 0,   /* no scenario macro */
    LQT_PRESET_CPU_DEFAULT = 1,/* CON + ISO1, the shipped SingleCell/TPORd.cc:33,35 */
    LQT_PRESET_CON = 2,        /* CON only */
    LQT_PRESET_LQT1 = 3,       /* LQT1 (GKs x0.05), no ISO */
    LQT_PRESET_GPU3D = 4,      /* LQT1 + ISO1 (PCa x4) + SUPREP 100 fmol, GPU3D.cu:18-22 */
    LQT_PRESET_GPU2D = 5       /* LQT1 only, new_11.cu:18-21 */
};
int lqt_model_preset(int preset, lqt_model *out);

/* Initial state of one cell (SingleCell/TPORd.cc:142-198), V0 replaced by v0
 * (-87.5 mV on the CPU, -86.2 mV in GPU3D.cu:213). */
int lqt_initial_state(double v0, double *state40_host);

/* ======================================================================== *
 *  Batched cells: N independent TPORd instances on the device.
 *  Replaces `new TPORd(ct)`, `setDt`, `setIstim`, `setDVgap_dt`, `update()`,
 *  `getV`, `getDvdt`, the current getters and `outputAllStates/readinAllStates`
 *  (SingleCell/TPORd.cc:137-376) for N cells at once.
 * ======================================================================== */
typedef struct lqt_cells lqt_cells;

/* types_host[n]: LQT_* cell type per cell.  stream: a cudaStream_t or NULL. */
int lqt_cells_create(int64_t n, const uint8_t *types_host, int precision,
                     const lqt_model *model, double dt, void *stream,
                     lqt_cells **out);
void lqt_cells_destroy(lqt_cells *c);
int64_t lqt_cells_count(const lqt_cells *c);

/* Whole state, n*40 doubles in reference order. */
int lqt_cells_set_state(lqt_cells *c, const double *state_host);
int lqt_cells_get_state(lqt_cells *c, double *state_host);

/* Per-cell stimulus (pA/pF) and gap-junction term dV/dt (mV/ms) held for the
 * following updates (setIstim / setDVgap_dt).  NULL sets all to zero. */
int lqt_cells_set_inputs(lqt_cells *c, const double *istim_host,
                         const double *dvgap_host);

/* nsteps calls of TPORd::update() on every cell (SingleCell/TPORd.cc:379-1021). */
int lqt_cells_update(lqt_cells *c, int64_t nsteps);

/* Membrane potential and dV/dt of the last update (getV, getDvdt). */
int lqt_cells_get_v(lqt_cells *c, double *v_host);
int lqt_cells_get_dvdt(lqt_cells *c, double *dvdt_host);

/* Currents of the last update, currents_host[n][6]: INa, ICaL, IKr, IKs, IK1
 * (pA/pF) and |dV/dt| (mV/ms) -- getINa, getICaL, getIKr, getIKs, getIK1,
 * getAbsDvdt (SingleCell/TPORd.cc:358-376).  Zero before the first update. */
int lqt_cells_get_currents(lqt_cells *c, double *currents_host);

/* Text state dump and restore of cells [first, first + count), cell after
 * cell on an open stream: outputAllStates writes each cell's 40 states as
 * "%4.10f\n" lines in the LQT_S_* order (SingleCell/TPORd.cc:200-252);
 * readinAllStates reads 40 "%lf" values per cell in the same order
 * (SingleCell/TPORd.cc:254-353).  The stream stays open and positioned after
 * the cells, so several calls (or other writes) can share one file, as the
 * reference's FILE* interface allows.  A read that runs out of values or finds
 * a non-number returns LQT_ERR_IO and leaves every cell's state unchanged. */
int lqt_cells_output_states(lqt_cells *c, int64_t first, int64_t count, FILE *f);
int lqt_cells_readin_states(lqt_cells *c, int64_t first, int64_t count, FILE *f);
/* The same text format for host state arrays (ncells x 40 doubles); no GPU. */
int lqt_state_write_text(const double *state40, int64_t ncells, FILE *f);
int lqt_state_read_text(double *state40, int64_t ncells, FILE *f);

/* ======================================================================== *
 *  Batches of independent instances: single cells and 1D strands, run to
 *  completion in one persistent launch.  Replaces the OneD.cc:100-436 strand
 *  loop (stimulus to the first cells, mirrored-end diffusion
 *  dVgap = dD/dx dV/dx + D d2V/dx2, update) and the SingleCell.cc:95-109 loop,
 *  for many instances with their own parameters at once.
 * ======================================================================== */
typedef struct lqt_batch lqt_batch;

typedef struct lqt_instance {
    int32_t ncells;            /* 1 = single cell; > 1 = strand (OneD.cc:100) */
    int32_t n_stim;            /* cells [0, n_stim) receive S1 (3 in OneD.cc:340) */
    int32_t model;             /* index into the models array */
    int32_t record;            /* 1 = record V every rec_every steps; strands also
                                  record the pseudo-ECG at ecg_x0; 3 = also ICaL
                                  and IKs of the first cell (SingleCell.cc:113-139) */
    double dx;                 /* mm (0.15, OneD.cc:47) */
    double bcl;                /* ms */
    double s1_start;           /* ms into each cycle */
    double s1_duration;        /* ms */
    double s1_strength;        /* pA/pF */
    int32_t s1_beats;          /* stimulated cycles; 0 = every cycle */
    int32_t reserved0;
    double t_stop;             /* steps run while time <= t_stop (OneD.cc:317) */
    double ecg_x0;             /* electrode, mm from cell 0 (35 in plot1DECG_compare.py:83) */
    double act_threshold;      /* mV (-30, OneD.cc:422) */
    /* S2 (OneD_VW.cc:265-279): cells [s2_cell0, s2_cell0 + s2_ncells) receive
     * s2_strength at the steps whose time t has t - s2_base >= s2_offset and
     * t - s2_base < s2_offset + s2_duration, unless an S1 window is open
     * (the reference tests S1 first).  s2_ncells = 0: no S2. */
    double s2_base, s2_offset, s2_duration, s2_strength;
    int32_t s2_cell0, s2_ncells;
    /* 1 = keep the maximum V of every cell over the steps with
     * t - s2_base >= s2_offset, starting from -100 (maxEndo / maxEpi,
     * OneD_VW.cc:246-247,340-344); read with lqt_batch_get_vmax. */
    int32_t track_vmax;
    int32_t reserved1;         /* must be zero */
} lqt_instance;

typedef struct lqt_batch_params {
    double dt;                 /* ms */
    double v0;                 /* initial V (-87.5, SingleCell/TPORd.cc:144) */
    int32_t precision;         /* LQT_FP64 or LQT_MIXED */
    int32_t max_beats;         /* detector slots per cell */
    int64_t rec_every;         /* steps between V records (10 in OneD.cc:402) */
    int32_t threads;           /* CTA width 128/256/512; 0 = autotuned */
    int32_t ctas;              /* persistent CTAs; 0 = resident CTAs x SMs */
    void *stream;              /* cudaStream_t, or NULL for an owned stream (the
                                  run is a CUDA graph, which cannot be captured
                                  on the legacy default stream) */
} lqt_batch_params;

/* cell_types: all cells, instance by instance (sum of ncells).
 * coeff: per-cell diffusion coefficient D (mm^2/ms) or NULL = 0.154
 * (OneD.cc:68); dD/dx is formed as OneD.cc:123-131 does. */
int lqt_batch_create(const lqt_batch_params *params, int32_t ninst,
                     const lqt_instance *inst, const uint8_t *cell_types_host,
                     const double *coeff_host, int32_t nmodels,
                     const lqt_model *models, lqt_batch **out);
void lqt_batch_destroy(lqt_batch *b);
int64_t lqt_batch_num_cells(const lqt_batch *b);
/* Run every instance to its t_stop (one persistent launch). */
int lqt_batch_run(lqt_batch *b);
/* Per cell (input order) and beat: activation time, APD90, max |dV/dt| of the
 * upstroke ([cells][max_beats], -1 = none), EAD flag and beats seen. */
int lqt_batch_get_detect(lqt_batch *b, float *t_act, float *apd90,
                         float *dvdt_max, uint8_t *ead, int32_t *nbeats);
/* Recorded V of instance i ([nrec][ncells]), record times and pseudo-ECG. */
int lqt_batch_get_record(lqt_batch *b, int32_t inst, double *v, double *t,
                         double *ecg, int64_t cap, int64_t *nrec);
/* ICaL and IKs of the first cell at the same records (record = 3). */
int lqt_batch_get_record_currents(lqt_batch *b, int32_t inst, double *ical,
                                  double *iks, int64_t cap, int64_t *nrec);
/* Per cell (input order): the maximum V of the track_vmax watch. */
int lqt_batch_get_vmax(lqt_batch *b, float *vmax_host);
int lqt_batch_get_state(lqt_batch *b, double *state_host);
int lqt_batch_set_state(lqt_batch *b, const double *state_host);
/* The launch configuration the autotuner chose (threads = 0 in the params):
 * CTA width, minimum resident CTAs/SM of the kernel variant, persistent CTAs
 * and the number of work items. */
int lqt_batch_config(const lqt_batch *b, int32_t *threads, int32_t *minb,
                     int32_t *ctas, int32_t *nitems);
/* Device time of the last run, ms (CUDA events on the batch stream). */
double lqt_batch_last_run_ms(const lqt_batch *b);
/* Blow-up counter of the last run (voxel-steps with NaN or V out of range). */
int64_t lqt_batch_num_bad(lqt_batch *b);

/* Last error message of the calling thread ("" if none). */
const char *lqt_last_error(void);

/* ======================================================================== *
 *  Tissue simulation: 1D strand, 2D sheet or 3D volume with diffusion.
 *  Replaces the OneD.cc:317-436 loop (1D) and the GPU3D.cu / new_11.cu
 *  kernel chain calc_du -> init_Istim -> set_Istim -> Itot -> new_u_v.
 * ======================================================================== */
typedef struct lqt_sim lqt_sim;

typedef struct lqt_geometry {
    int32_t nx, ny, nz;        /* grid; 1D strand: ny = nz = 1 */
    double dx;                 /* mm */
    const uint8_t *cell_type;  /* nx*ny*nz host array, LQT_* or LQT_EMPTY; index
                                  (x*ny + y)*nz + z (x-major, as GPU3D.cu:1307-1333) */
    const float *fibre;        /* nx*ny*nz*3 unit fibre vectors, or NULL = isotropic */
    double d_fibre;            /* mm^2/ms along fibres (isotropic value when fibre == NULL) */
    double d_trans;            /* mm^2/ms across fibres */
    const double *coeff_1d;    /* 1D only: per-cell D (OneD.cc:103-131), or NULL = d_fibre */
} lqt_geometry;

typedef struct lqt_protocol {
    double bcl;                /* ms */
    double s1_start;           /* ms into each cycle (OneD.cc:81) */
    double s1_duration;        /* ms */
    double s1_strength;        /* pA/pF */
    int32_t s1_beats;          /* number of S1 cycles stimulated; 0 = every cycle */
    int32_t reserved0;
    const uint8_t *s1_mask;    /* nx*ny*nz host array: 1 = receives S1 */
    const float *s1_onset;     /* optional per-voxel onset delay, ms (GPU3D.cu:397-409) */
    double s2_time;            /* absolute ms; < 0 = no S2 */
    double s2_duration;
    double s2_strength;
    const uint8_t *s2_mask;    /* nx*ny*nz host array: 1 = receives S2 */
} lqt_protocol;

/* A NULL stream makes the simulation create and own a non-blocking stream
 * (graph capture cannot use the legacy default stream). */
typedef struct lqt_sim_params {
    double dt;                 /* ms (0.02 in every reference driver) */
    double v0;                 /* initial V, mV */
    int32_t precision;         /* LQT_FP64 or LQT_MIXED */
    int32_t detect;            /* 1 = on-device activation / APD90 / EAD detectors */
    lqt_model model;
    double act_threshold;      /* mV, activation crossing (-30, OneD.cc:422) */
    double vmin_ok, vmax_ok;   /* blow-up detector range (GPU3D.cu:1805-1817 warns below
                                  -90 / above 200); vmin_ok >= vmax_ok = NaN check only */
    void *stream;              /* cudaStream_t or NULL */
} lqt_sim_params;

int lqt_sim_create(const lqt_sim_params *params, const lqt_geometry *geom,
                   lqt_sim **out);
void lqt_sim_destroy(lqt_sim *s);
int lqt_sim_set_protocol(lqt_sim *s, const lqt_protocol *p);

/* Tissue voxel count and the dense grid index of each tissue voxel (the
 * reference's rev_g, GPU3D.cu:1323). */
int64_t lqt_sim_num_tissue(const lqt_sim *s);
int lqt_sim_tissue_index(const lqt_sim *s, int64_t *grid_index_host);

/* Advance nsteps of dt.  Simulated time accumulates as `time += dt` in FP64,
 * as the reference drivers do (OneD.cc:317).  Returns when the steps have run
 * on the device. */
int lqt_sim_step(lqt_sim *s, int64_t nsteps);
/* The same steps, enqueued on the simulation's stream without waiting: a host
 * loop that issues one step at a time (with a read-back per step) keeps the
 * device busy instead of paying a host round-trip per step.  Device errors
 * surface at the next call that waits (lqt_sim_sync, lqt_sim_step, a read). */
int lqt_sim_step_async(lqt_sim *s, int64_t nsteps);
/* Waits for every step enqueued on the simulation's stream. */
int lqt_sim_sync(lqt_sim *s);
double lqt_sim_time(const lqt_sim *s);

/* V of every tissue voxel (tissue order), as float or double. */
int lqt_sim_get_v(lqt_sim *s, void *v_host, int as_double);
/* Whole state, ntissue*40 doubles in reference order. */
int lqt_sim_get_state(lqt_sim *s, double *state_host);
int lqt_sim_set_state(lqt_sim *s, const double *state_host);

/* Pseudo-ECG electrodes (mm, grid frame).  The value at an electrode r0 is
 * sum_i sum_axis (V[i+e]-V[i-e])/2 * (r_i - r0)_axis / |r_i - r0|^3, the 3D
 * form of PlotScript/plot1DECG_compare.py:89-105.  Sampled every `every` steps. */
int lqt_sim_set_electrodes(lqt_sim *s, int32_t n, const double *xyz_host,
                           int32_t every);
/* V of every tissue voxel into a host buffer without waiting (the reference
 * copies V back every step, GPU3D.cu:1802): the gather into one of 16 device
 * slots runs on the simulation's stream, the copy on four copy streams, so it
 * overlaps the next steps; the steps wait only when all 16 slots hold copies
 * still in flight.  The first call allocates the slots (16 x ntissue x 8
 * bytes of device memory, kept until lqt_sim_destroy).  The copies of one simulation are numbered 0, 1, ... in
 * call order (the first call after lqt_sim_create is copy 0) and complete in
 * that order.  The buffer (pinned memory for a true overlap) is complete after
 * lqt_sim_wait_v_upto(its number) or lqt_sim_wait_v, and must not be reused
 * before. */
int lqt_sim_get_v_async(lqt_sim *s, void *v_host, int as_double);
/* Waits for every read-back copy in flight. */
int lqt_sim_wait_v(lqt_sim *s);
/* Waits for read-back copies 0..seq (seq < the number of copies issued).  A
 * caller that reads V back every step keeps a ring of host buffers and waits
 * for the copy that last filled a buffer before reusing it: the host then
 * never waits on the newest copy, and the GPU never idles on the host. */
int lqt_sim_wait_v_upto(lqt_sim *s, int64_t seq);

/* Samples recorded since the electrodes were set: [nsamples][n], and time. */
int lqt_sim_get_ecg(lqt_sim *s, int64_t max_samples, double *phi_host,
                    double *t_host, int64_t *nsamples);

/* Detector results per tissue voxel (detect = 1): last activation time (ms,
 * first upward crossing of act_threshold in a cycle, OneD.cc:419-436), APD90
 * of the last completed beat (ms from activation to the first step at or
 * below overshoot - 0.9 * (overshoot - rest), the amplitude rule of
 * SingleCell.cc:185-212, with the overshoot taken as the maximum V since
 * activation: in tissue an upstroke can stall for one step where waves
 * collide, and the single-cell "first non-rising step" would then depend on
 * microvolt differences) and an EAD flag (a rise of V after the 50% level,
 * before 90% repolarisation).  NULL pointers are skipped. */
int lqt_sim_get_detect(lqt_sim *s, float *t_act_host, float *apd90_host,
                       uint8_t *ead_host);

/* Occupancy variant of the fused step kernel: the minimum resident CTAs/SM its
 * register allocation allows (mixed form 2, 3, 4; FP64 1, 2).  variant >= 0
 * forces one; variant < 0 runs the autotuner now (15 real steps, the variants
 * in turn, each timed with CUDA events, the fastest kept; with a surrogate
 * attached, 15 more steps pick the variant of the V-only substep kernel).  The
 * first lqt_sim_step call with nsteps >= 64 autotunes by itself unless a
 * variant was forced.  All variants give bit-identical results.
 * ms_per_variant: up to 4 timings (or NULL). */
int lqt_sim_tune(lqt_sim *s, int32_t variant, int32_t *chosen, float *ms_per_variant);

/* Kernel of the V-only substep inside a surrogate macro step: 5, 6, 8 = one
 * thread per voxel with direct loads, at that many CTAs/SM; 105, 106, 108 =
 * persistent CTAs that stage each 256-voxel tile's streamed rows (rate, index,
 * tensor, control, detector flag) in shared memory with bulk asynchronous
 * copies, two tiles in flight, at 5, 6, 8 CTAs/SM (2D/3D anisotropic grids;
 * elsewhere the direct kernel runs); 203, 204 = the same with each tile's
 * V halo (the box of the dense V grid its 19-point stencils reach, copied as
 * z-segments of its columns) staged in shared memory too, at 3, 4 CTAs/SM
 * (3D anisotropic grids with nz a multiple of 4; elsewhere 105 runs);
 * 304, 305, 306 = one producer warp streams each tile's rows into a two-stage
 * shared-memory ring (full/empty barriers) while eight warps compute, V read
 * from the grid, at 4, 5, 6 CTAs/SM (2D/3D anisotropic grids; elsewhere 105
 * runs).  variant >= 0 forces one (the autotuner then keeps it); variant < 0
 * only reports the current one.  All variants give bit-identical results.
 * ms_per_variant (or NULL): 11 mean milliseconds per step from the last
 * autotune, in the order 5, 6, 8, 105, 106, 108, 203, 204, 304, 305, 306
 * (zeros if it has not run). */
int lqt_sim_substep_variant(lqt_sim *s, int32_t variant, int32_t *chosen, float *ms_per_variant);

/* Instrumentation (no counterpart in the reference, which has no timing):
 * run nsteps steps without graph capture, timing each launch of the fused
 * step kernel, of the ghost/clock kernel and (with a surrogate attached) of
 * the surrogate macro-step kernel with CUDA events on the simulation's
 * stream; returns the mean milliseconds per launch (ms_sur: per macro-step
 * launch, 0 when none ran).  NULL outputs are skipped. */
int lqt_sim_profile(lqt_sim *s, int64_t nsteps, double *ms_step, double *ms_ghost,
                    double *ms_sur);

/* Mirror-boundary map (GPU3D.cu:1487-1604): the empty grid voxels next to
 * tissue and, for each, the grid index of the tissue voxel whose V it holds.
 * Call with dst = src = NULL to get the count. */
int lqt_sim_boundary(const lqt_sim *s, int64_t *dst_host, int64_t *src_host,
                     int64_t *n);

/* Pseudo-ECG of a caller-owned V grid that allocates nothing (no counterpart
 * in the reference).  For callers that cannot call cudaMalloc: a host framework
 * that owns all device memory and hands out fixed buffers, or a stepping loop
 * that must not take the device-wide synchronisation of cudaMalloc/cudaFree.
 * Same sum as lqt_sim_set_electrodes / lqt_sim_get_ecg.  v_grid_dev: FP32 V of
 * the nx*ny*nz grid, x-major: voxel (x, y, z) at index (x*ny + y)*nz + z, with
 * the empty voxels next to tissue holding their mirror source's V (1D: the
 * strand itself, ny = nz = 1); tissue_index_dev: int32 grid index of each
 * tissue voxel (NULL for 1D); positions are in the grid frame with voxel
 * (x, y, z) at (x*dx, y*dx, z*dx) mm (origin at voxel 0, no offset);
 * electrodes_host: nel*3 mm in that frame; phi_dev: nel doubles written on
 * `stream`.  Precondition (2D/3D): no tissue voxel on a grid face, i.e.
 * 1 <= x <= nx-2, 1 <= y <= ny-2 and, in 3D, 1 <= z <= nz-2.  The kernel
 * checks every index before it reads V: a voxel that breaks this is skipped
 * and every phi becomes NaN (the call is asynchronous, so this is how a bad
 * index is reported; nothing outside the grid is read).
 * Limits: 1 <= nel <= 8; ntissue and the grid below 2^31.  Its scratch is a
 * fixed device array inside the library, 128 KiB of partials plus a 256-byte
 * status word (every GPU that loads the library holds it until exit); the
 * first call on a device looks up that array's address, so make it before any
 * stream capture.  The address is cached per device for the process; after a
 * cudaDeviceReset the first call's launch fails with LQT_ERR_CUDA and drops
 * the cached address, and the next call looks it up again.  Calls that
 * overlap on the GPU share the array and race: serialise them. */
int lqt_ecg_grid_noalloc(const float *v_grid_dev, int32_t nx, int32_t ny,
                         int32_t nz, double dx, const int32_t *tissue_index_dev,
                         int64_t ntissue, const double *electrodes_host,
                         int32_t nel, double *phi_dev, void *stream);

/* Blow-up detector: count of voxels with NaN or V outside [vmin_ok, vmax_ok]
 * since the last call (GPU3D.cu:1796-1829 does this scan on the host);
 * LQT_ERR_NUMERIC when it is not zero.  Also LQT_ERR_CUDA when a surrogate
 * substep's tile-copy wait ran out (some voxels missed a substep). */
int lqt_sim_check(lqt_sim *s, int64_t *n_bad);

/* Binary checkpoint: header + version + per-state arrays. */
int lqt_sim_checkpoint(lqt_sim *s, const char *path);
int lqt_sim_restore(lqt_sim *s, const char *path);

/* ======================================================================== *
 *  Output files in the reference drivers' formats.
 * ======================================================================== */

/* V on the lattice of every `stride`-th voxel per axis of a 2D/3D grid, in
 * the order the reference's VTK writer visits it (z outermost, x innermost),
 * -100 where the grid voxel is not tissue (GPU3D.cu:145-158 with stride 3,
 * new_11.cu:164-175 with stride 1).  Sampled on the device.  out_host = NULL
 * returns the count in *n. */
int lqt_sim_sample_v(lqt_sim *s, int32_t stride, double *out_host, int64_t cap,
                     int64_t *n);

/* Legacy-VTK structured-points file of such samples, byte for byte the file
 * of GPU3D.cu:123-163 / new_11.cu:142-180: header with DIMENSIONS
 * nx/stride ny/stride nz/stride (integer division), values printed as a C++
 * stream prints a double ("%g"), each followed by a space, a newline after
 * every x row and after every z plane. */
int lqt_io_write_vtk(const char *path, const double *samples_host, int32_t nx,
                     int32_t ny, int32_t nz, int32_t stride);

/* Rows of "%4.10f\t" values, each row ended by a newline: the .dat files of
 * OneD.cc:402-415 (time, V of each cell), SingleCell.cc:113-139 (time, V,
 * ICaL, IKs) and OneD_VW.cc (V of each cell).  append != 0 appends. */
int lqt_io_write_dat(const char *path, int64_t nrows, int32_t ncols,
                     const double *rows_host, int32_t append);

/* Input files of the reference drivers.
 * Geometry: one line per tissue voxel, "x y z fx fy fz code" (dim 3,
 * GPU3D.cu:1276-1296,1424-1468) or "x y fx fy code" (dim 2,
 * new_11.cu:1296-1302,1444-1478), into x-major grids of nx*ny*nz voxels (z
 * fastest; nz = 1 in 2D): cell_type (codes 7-10, 17-20 -> LQT_EPI; 4-6,
 * 14-16 -> LQT_MCELL; other codes -> LQT_ENDO; LQT_EMPTY where no line),
 * code (the file's code after the edits, 0 elsewhere), fibre (3 floats per
 * voxel; fz = 0 in 2D) and s2_mask.  case_edits = 1 applies the reference's
 * case-study edits: 3D, RV M cells (codes 4-6) become code 2 if fy <= 4 else
 * 7, LV M cells (14-16) outside 75 voxels of (597, 336, 336) become 12 (code
 * 14) or 17, S2 box x in [300, 687), y in [120, 486), z in [420, 534)
 * (GPU3D.cu:1437-1466); 2D, codes 3-6 become 2 (<= 4) or 7, LV M cells
 * (13-16) outside x in [550, 689), y in [150, 487) become 12 or 17, S2 where
 * x in [300, 400), y in [200, 350) and the original code is 11-13
 * (new_11.cu:1452-1478).  Output arrays may be NULL.  Blank lines are
 * skipped; a point outside the grid or a repeated point is an error. */
typedef struct lqt_geom_file_spec {
    int32_t dim;
    int32_t nx, ny, nz;
    int32_t case_edits;
    int32_t reserved;          /* must be zero */
} lqt_geom_file_spec;
int lqt_io_read_geometry(const char *path, const lqt_geom_file_spec *spec,
                         uint8_t *cell_type, uint8_t *code, float *fibre,
                         uint8_t *s2_mask, int64_t *ntissue);
/* Stimulation profile "x y z a b c onset tag" (GPU3D.cu:1694-1712): points
 * that are tissue in cell_type get s1_mask = 1 and their onset (ms, read as
 * float).  layer >= 0 (2D): only lines with z == layer, mapped to (x, y)
 * (new_11.cu:1723-1741 uses layer 157).  Points off the grid or off tissue
 * are skipped, as the reference skips them. */
int lqt_io_read_stimulation(const char *path, int32_t nx, int32_t ny, int32_t nz,
                            int32_t layer, const uint8_t *cell_type,
                            uint8_t *s1_mask, float *onset, int64_t *npoints);

/* Asynchronous VTK snapshots of a simulation: submit() samples V on the
 * device and copies it into one of nbuf pinned buffers on the simulation's
 * stream, then returns; a host thread writes the file once the copy is done
 * (submit waits only when all buffers are in flight).  flush() waits for
 * every pending file and reports the first write error.  The simulation must
 * outlive the writer. */
typedef struct lqt_vtk_writer lqt_vtk_writer;
int lqt_vtk_writer_create(lqt_sim *s, int32_t stride, int32_t nbuf,
                          lqt_vtk_writer **out);
int lqt_vtk_writer_submit(lqt_vtk_writer *w, const char *path);
int lqt_vtk_writer_flush(lqt_vtk_writer *w);
void lqt_vtk_writer_destroy(lqt_vtk_writer *w);

/* ======================================================================== *
 *  Learned surrogate network (no counterpart in the reference): MLP
 *  48 -> 128 -> 128 -> 48 with SiLU, BF16 weights, FP32 accumulation.
 *  Parameters are one FP32 block of lqt_mlp_num_params() floats:
 *  W1 [128][48], b1 [128], W2 [128][128], b2 [128], W3 [48][128], b3 [48]
 *  (weights [out][in]).  Inference and the training GEMMs (forward, backward
 *  and weight gradients) run on the tcgen05 tensor cores with the
 *  accumulators in TMEM; every tensor-core completion wait is bounded and a
 *  wait that runs out makes the next call that waits return LQT_ERR_TIMEOUT.
 *  Device buffers belong to the caller.
 * ======================================================================== */
typedef struct lqt_mlp lqt_mlp;
int lqt_mlp_create(uint64_t seed, void *stream, lqt_mlp **out);
void lqt_mlp_destroy(lqt_mlp *m);
int64_t lqt_mlp_num_params(void);
int lqt_mlp_set_params(lqt_mlp *m, const float *params_host);
/* Parameters and the gradients of the last gradient/training call (NULL skips). */
int lqt_mlp_get_params(lqt_mlp *m, float *params_host, float *grads_host);
/* Feature normalisation: x_n = (x - in_mean) * in_scale; state change =
 * y * out_scale; nvalid = outputs that carry a target (<= 48). */
int lqt_mlp_set_norm(lqt_mlp *m, const float *in_mean, const float *in_scale,
                     const float *out_scale, int32_t nvalid);
/* Residual bounds of the surrogate (48 values > 0, normalised output units):
 * a tissue macro step accepts a voxel only if every normalised correction
 * |y_j| <= kappa * out_bound[j] (lqt_sur_config.kappa); typically the largest
 * |target| of the training set.  Default: unbounded. */
int lqt_mlp_set_bounds(lqt_mlp *m, const float *out_bound);
/* Shared-memory descriptor stride assignment used by the tensor-core
 * kernels: 0 = leading offset along K (default), 1 = swapped (diagnostic). */
int lqt_mlp_set_layout(lqt_mlp *m, int32_t layout);
/* y[n][48] = MLP(x[n][48]); x BF16, y FP32, both device pointers. */
int lqt_mlp_infer(lqt_mlp *m, const void *x_bf16_dev, float *y_dev, int64_t n);
/* Loss = mean over the nvalid outputs of (y - t)^2 and its gradients for a
 * batch (multiple of 16) of device inputs (BF16) and targets (FP32). */
int lqt_mlp_gradients(lqt_mlp *m, const void *x_bf16_dev, const float *t_dev,
                      int64_t batch, double *loss);
/* lqt_mlp_gradients followed by one Adam step (beta 0.9 / 0.999). */
int lqt_mlp_train_step(lqt_mlp *m, const void *x_bf16_dev, const float *t_dev,
                       int64_t batch, float lr, double *loss);

/* Training pairs for the surrogate from the plain mixed-form integrator:
 * ncells paced cells with seeded uniform parameters in the given ranges
 * (GKs factor, PCa factor, GKs-ISO factor, BCL; type uniform over
 * endo/M/epi; 2 ms x -52 pA/pF at 50 ms of each cycle).  After beats_warm
 * cycles, at macro-step boundaries (every nsub steps) where |dV/dt| <=
 * dvdt_max and no stimulus falls in the coming macro step, each cell records
 * with probability prob: x_dev[row][44] = 38 states (V, 8 concentrations, 29
 * gates) + 3 factors + endo/epi/M one-hot, d_dev[row][38] = the state after
 * nsub plain steps of dt minus the state after one coarse step of nsub * dt
 * from the same start (the correction the network learns).  Macro steps that are not
 * recorded carry a seeded constant current uniform in +-jitter pA/pF, which
 * moves the cells off the single-cell trajectory as tissue coupling does.
 * Up to cap rows; *count = rows written.  The rows are in cell order (cell
 * after cell, each cell's pairs in time order; a set longer than cap keeps the
 * first cells), so the same arguments give the same bits on every run. */
typedef struct lqt_sur_ranges {
    double gks[2], pca[2], iso[2], bcl[2];
    int32_t beats_warm, beats_record;
    double dt, dvdt_max, prob, jitter;
    int32_t nsub;       /* plain steps per macro step; divides 50; 0 = 5 */
    int32_t reserved;   /* must be zero */
} lqt_sur_ranges;
int lqt_sur_datagen(int64_t ncells, uint64_t seed, const lqt_sur_ranges *ranges,
                    float *x_dev, float *d_dev, int64_t cap, int64_t *count,
                    void *stream);
/* Rows idx_dev[n] (or 0..n-1 when NULL) of raw features / changes -> the
 * network's normalised BF16 inputs xb_dev[n][48] and FP32 targets t_dev[n][48]
 * (d_dev may be NULL for inputs only). */
int lqt_sur_prepare(lqt_mlp *m, const float *x_dev, const float *d_dev,
                    const int64_t *idx_dev, int64_t n, void *xb_dev, float *t_dev);

/* The surrogate inside a tissue simulation (mixed form only).  Every nsub
 * steps (steps whose index is a multiple of nsub; nsub divides 50, 0 = 5)
 * one kernel offers each tissue voxel whose |dV/dt| over the last step is at
 * most dvdt_max, that is not at the foot of a wave (foot_dvdt, foot_v), and
 * that no stimulus reaches in the next nsub steps, to the
 * surrogate: one coarse TPORd step of nsub * dt plus the network's
 * correction (use_net = 1; 0 = the coarse step alone).  The residual check (every normalised correction within
 * +-kappa times its bound, lqt_mlp_set_bounds; gates within [0, 1];
 * concentrations positive; ionic V change of the macro step within
 * +-vstep_max mV) decides per voxel; a voxel that
 * passes keeps its new ionic state and, for the next nsub steps, moves V by the
 * macro step's ionic rate plus diffusion only.  Every other voxel runs the
 * plain step.  The network must be trained for this dt and nsub (training
 * pairs from lqt_sur_datagen with the same dt and nsub); its inputs carry the model's GKs, PCa and
 * GKs-ISO factors, so models with ISO gate shifts or a SUPREP dose are
 * refused.  m = NULL detaches.  m stays owned by
 * the caller and must outlive the attachment; its parameters are read at
 * every macro step. */
typedef struct lqt_sur_config {
    double dvdt_max;    /* mV/ms, e.g. 1.5 */
    double kappa;       /* multiplier of the network's residual bounds, e.g. 1.5 */
    double vstep_max;   /* mV per macro step, e.g. 0.4 */
    int32_t use_net;
    int32_t nsub;       /* plain steps per macro step; divides 50; 0 = 5 */
    /* wave-foot gate: a voxel below foot_v (mV) whose V rose faster than
     * foot_dvdt (mV/ms) over the last step is not offered -- the foot of an
     * approaching wave, where diffusion drives V towards threshold and an
     * ionic state advanced without it would delay the upstroke.  foot_dvdt
     * = 0 turns the gate off (then |dV/dt| <= dvdt_max alone decides). */
    double foot_dvdt;   /* mV/ms, e.g. 0.1 (the Python default) */
    double foot_v;      /* mV, e.g. -40 */
} lqt_sur_config;
int lqt_sim_set_surrogate(lqt_sim *s, lqt_mlp *m, const lqt_sur_config *cfg);
/* Counters since the last reset: macro steps launched, voxel offers, voxels
 * accepted; wait_timeouts: bit 0 set if a tensor-core completion wait of the
 * macro step ran out (the affected voxels ran the plain step), bit 1 if a
 * tile-copy wait of the staged substep ran out (that CTA's remaining voxels
 * missed the substep: the run is not valid).  reset != 0 zeroes them. */
int lqt_sim_surrogate_stats(lqt_sim *s, int64_t *macro_steps, int64_t *offered,
                            int64_t *accepted, int32_t *wait_timeouts, int32_t reset);
/* Offered voxels that failed each residual check since the last reset (a voxel
 * can fail several): counts[0] a normalised correction beyond kappa times its
 * bound, [1] a gate outside [0, 1] or not finite, [2] a concentration not
 * positive, [3] the ionic V change beyond vstep_max. */
int lqt_sim_surrogate_rejections(lqt_sim *s, int64_t *counts);
/* Test of the failure path, no use in production runs: skip_first_copy = 1
 * makes the staged substep kernel (variants 105/106/108) leave out the first
 * tile's copies of every CTA, so that tile's bounded mbarrier wait runs out;
 * wait_limit sets the polls per wait (0 = the default).  The CTA then sets bit
 * 1 of the surrogate error word, lets its copies in flight land and returns;
 * lqt_sim_check reports it and the context stays usable.  (0, 0) restores. */
int lqt_sim_set_wait_test(lqt_sim *s, int32_t skip_first_copy, uint32_t wait_limit);

/* ======================================================================== *
 *  Synthetic geometries (seeded).  The reference reads its geometry from
 *  files that are not distributed (wholeventriclewithfibervector.txt,
 *  157layerwithfibervector.txt, GPU3D.cu:1276, new_11.cu:1296); these
 *  generators produce grids in the same layout (x-major, z fastest).
 * ======================================================================== */

/* 2D sheet of nx*ny tissue voxels in a grid of (nx+2)*(ny+2) (one empty
 * voxel on each side; all arrays have the grid's size): types in bands along
 * x (frac_endo endo, frac_mid M, rest epi); s1_mask = first s1_cols tissue
 * columns; s2_mask = tissue quadrant x < nx/2, y < ny/2.  Masks may be NULL. */
int lqt_geom_sheet(int32_t nx, int32_t ny, double frac_endo, double frac_mid,
                   int32_t s1_cols, uint8_t *types, uint8_t *s1_mask,
                   uint8_t *s2_mask);

/* Truncated prolate-ellipsoid shell (all lengths mm): outer semi-axes a_out
 * (x, y) and c_out (z), wall thickness `wall`, axis at (cx, cy), base plane
 * z = z_base (tissue below it), apex at z_base - c_out.  Transmural depth
 * e in [0,1] (endo -> epi): endo for e < endo_frac, epi for e >= 1 - epi_frac;
 * between them M cells inside a seeded spherical island of island_radius in
 * the free wall (centre returned in island_out[3]), endo/epi outside it (as
 * GPU3D.cu:1440-1461 cancels M cells outside its island).  Fibre angle
 * linear in e from alpha_endo_deg to alpha_epi_deg, measured from the
 * circumferential direction towards the meridian.  s1_mask: tissue within
 * stim_radius of the apex. */
typedef struct lqt_ventricle_spec {
    int32_t nx, ny, nz;
    int32_t reserved0;
    double dx;
    double a_out, c_out, wall;
    double cx, cy, z_base;
    double endo_frac, epi_frac;
    double island_radius;
    double alpha_endo_deg, alpha_epi_deg;
    double stim_radius;
    uint64_t seed;
} lqt_ventricle_spec;

int lqt_geom_ventricle(const lqt_ventricle_spec *spec, uint8_t *types,
                       float *fibre, uint8_t *s1_mask, double *island_out);

/* Host-only tissue numbering and mirror-boundary map of a grid (what
 * lqt_sim_create builds; GPU3D.cu:1307-1333, 1487-1604; new_11.cu:1535-1640).
 * tissue_of[nx*ny*nz]: tissue index or -1.  bnd_dst/bnd_src: boundary voxel
 * and its mirror source (grid indices); NULL to query *nbnd first. */
int lqt_geom_mirror_map(int32_t nx, int32_t ny, int32_t nz,
                        const uint8_t *types, int32_t *tissue_of,
                        int64_t *bnd_dst, int64_t *bnd_src, int64_t *nbnd);
/* The same numbering and mirror-boundary map built on the GPU (one thread per
 * grid voxel, then an ordered compaction), bit-identical to the host builder;
 * lqt_sim_create uses it.  Host arrays in and out, as lqt_geom_mirror_map;
 * stream: a cudaStream_t or NULL.  Grid below 2^31 voxels. */
int lqt_geom_mirror_map_gpu(int32_t nx, int32_t ny, int32_t nz,
                            const uint8_t *types, int32_t *tissue_of,
                            int64_t *bnd_dst, int64_t *bnd_src, int64_t *nbnd,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif /* LQT_H_ */
