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
 *  `getV`, `outputAllStates/readinAllStates` (SingleCell/TPORd.cc:137-376)
 *  for N cells at once.
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

typedef struct lqt_sim_params {
    double dt;                 /* ms (0.02 in every reference driver) */
    double v0;                 /* initial V, mV */
    int32_t precision;         /* LQT_FP64 or LQT_MIXED */
    int32_t detect;            /* 1 = on-device activation / APD90 / EAD detectors */
    lqt_model model;
    double act_threshold;      /* mV, activation crossing (-30, OneD.cc:422) */
    double vmin_ok, vmax_ok;   /* blow-up detector range (GPU3D.cu:1805-1817: -90/200 warn) */
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
 * as the reference drivers do (OneD.cc:317). */
int lqt_sim_step(lqt_sim *s, int64_t nsteps);
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
/* Samples recorded since the electrodes were set: [nsamples][n], and time. */
int lqt_sim_get_ecg(lqt_sim *s, int64_t max_samples, double *phi_host,
                    double *t_host, int64_t *nsamples);

/* Detector results per tissue voxel (detect = 1): last activation time (ms,
 * first upward crossing of act_threshold in a cycle, OneD.cc:419-436), APD90
 * of the last completed beat (ms from activation; amplitude rule of
 * SingleCell.cc:185-212) and an EAD flag (second upstroke above -60 mV before
 * 90% repolarisation).  NULL pointers are skipped. */
int lqt_sim_get_detect(lqt_sim *s, float *t_act_host, float *apd90_host,
                       uint8_t *ead_host);

/* Blow-up detector: count of voxels with NaN or V outside [vmin_ok, vmax_ok]
 * since the last call (GPU3D.cu:1796-1829 does this scan on the host). */
int lqt_sim_check(lqt_sim *s, int64_t *n_bad);

/* Binary checkpoint: header + version + per-state arrays. */
int lqt_sim_checkpoint(lqt_sim *s, const char *path);
int lqt_sim_restore(lqt_sim *s, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* LQT_H_ */
