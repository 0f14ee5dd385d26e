/*
 * lqt_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the reference's TPORd path (ShugangZhang/LQT1),
 * used as the parity checker for the CUDA kernels and as the timed CPU
 * baseline.  Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it; the product library never links or calls it.
 *
 * Each function cites the reference lines it follows.  The single-cell update
 * keeps the reference's evaluation order expression by expression, so that
 * built with the same flags (-O3, no FP contraction) it reproduces the
 * reference's own TPORd::update() bit for bit; that is checked against the
 * reference built from its sources (oracle/build_ref.sh) and against golden
 * vectors in tests/golden/.
 */
#ifndef LQT_ORACLE_H_
#define LQT_ORACLE_H_

#include <stdint.h>
#include "../include/lqt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Currents reported by the reference getters (TPORd.cc:363-375). */
typedef struct orc_aux {
    double dvdt;     /* dV_dt = -(Iion + Ist), TPORd.cc:928 */
    double iion;
    double ina, inal, ito, ical, ikr, iks, ik1, inaca, inak;
} orc_aux;

/* SingleCell/TPORd.cc:142-198 */
void orc_initial_state(double v0, double *s);

/* One TPORd::update() (SingleCell/TPORd.cc:379-1021) of one cell.
 * s: 40 states in reference order; ctype: LQT_* cell type. */
void orc_update(double *s, int ctype, const lqt_model *m, double dt,
                double ist, double dvgap, orc_aux *aux);

/* n independent cells, nsteps updates each, OpenMP over cells. */
void orc_cells_update(int64_t n, double *s, const uint8_t *ctype,
                      const lqt_model *m, double dt, const double *ist,
                      const double *dvgap, int64_t nsteps, int nthreads);
/* The same updates, then the current getters of the last one, cur[n][6]:
 * INa, ICaL, IKr, IKs, IK1, |dV/dt| (SingleCell/TPORd.cc:358-376). */
void orc_cells_currents(int64_t n, double *s, const uint8_t *ctype,
                        const lqt_model *m, double dt, const double *ist,
                        const double *dvgap, int64_t nsteps, double *cur);

/* SingleCell.cc:95-232: single cell paced at bcl for nbeats; APD statistics of
 * the last beat.  stats out: [rest, dvdt_max, overshoot, amplitude, apd20,
 * apd25, apd50, apd75, apd80, apd90].  trace (optional): V after each step with
 * index step % trace_every == 0, up to trace_cap values; returns count. */
int64_t orc_single_cell_run(int ctype, const lqt_model *m, double v0,
                            double dt, double bcl, double nbeats,
                            double stim_start, double stim_dur,
                            double stim_strength, double *stats,
                            int64_t trace_every, double *trace,
                            int64_t trace_cap, double *final_state);

/* OneD.cc:100-436: strand of n cells, per-cell types and diffusion coefficient,
 * stimulus to cells [0, n_stim), time loop `time <= stop_time`.
 * rec: V of all cells after each step with step % rec_every == 0
 *      ([nrec][n], plus rec_t[nrec]); returns the number recorded.
 * act: per cell, activation times (first V >= act_thr after being below it),
 *      up to max_beats per cell ([n][max_beats], -1 = none).
 * cv_out: [cv, cv_start, cv_end] for cells 10 and 90 on the last S1 cycle
 *      (OneD.cc:419-436), NaN if the strand is shorter.
 * final_state: n*40 (optional). */
typedef struct orc_strand_cfg {
    int32_t n;
    double dx, dt;
    double bcl, stim_start, stim_dur, stim_strength;
    int32_t n_stim;
    int32_t num_s1;           /* cycles before the CV cycle (OneD.cc:77) */
    double stop_time;         /* OneD.cc:78 */
    double act_thr;           /* -30 mV */
} orc_strand_cfg;

int64_t orc_strand_run(const orc_strand_cfg *cfg, const uint8_t *ctype,
                       const double *coeff, const lqt_model *m, double v0,
                       int64_t rec_every, double *rec, double *rec_t,
                       int64_t rec_cap, int32_t max_beats, double *act,
                       double *cv_out, double *final_state, int nthreads);

/* One trial of the S1-S2 vulnerable-window search, OneD_VW.cc:199-349: a
 * fresh strand; S1 on cells [0, n_stim) in the window of every cycle
 * (stim_start, stim_dur, stim_strength); otherwise S2 on cells
 * [s2_cell0, s2_cell0 + s2_ncells) while t - (num_s1 - 1) * bcl is in
 * [s2_time, s2_time + s2_dur); steps while t <= stop_time.  Out: the
 * maximum V of the first and the last cell over the steps with
 * t - (num_s1 - 1) * bcl >= s2_time, starting at -100 (maxEndo, maxEpi), and
 * optionally V of every cell every 50 steps of cycle num_s1 - 1 (the
 * Transmural1D file rows).  Returns the rows written. */
int64_t orc_vw_trial(const orc_strand_cfg *cfg, const uint8_t *ctype,
                     const double *coeff, const lqt_model *m, double v0,
                     double s2_time, double s2_dur, double s2_strength,
                     int32_t s2_cell0, int32_t s2_ncells, double *max_endo,
                     double *max_epi, double *rec, int64_t rec_cap);

/* AP detector per cell and cycle, the definition the device kernels use:
 * on the step where a cycle's S1 window opens, rest = V before that step; an
 * upward crossing of act_thr marks activation; the upstroke ends at the first
 * step whose V is not above the previous V (overshoot = previous V,
 * SingleCell.cc:160-198); APD90 = time of the first step at or below
 * overshoot - 0.9 (overshoot - rest) minus the activation time; an EAD is a
 * rise of more than 1e-3 mV in one step after V fell below the 50% level and
 * before the 90% crossing.  Outputs per cell: t_act/apd90 per beat
 * ([n][max_beats], -1 = none), ead flag, beats opened. */
int64_t orc_strand_detect(const orc_strand_cfg *cfg, int32_t s1_beats,
                          const uint8_t *ctype, const double *coeff,
                          const lqt_model *m, double v0, int32_t max_beats,
                          double *t_act, double *apd90, uint8_t *ead,
                          int32_t *nact, double *final_state);

/* Pseudo-ECG of a strand (PlotScript/plot1DECG_compare.py:89-105). */
double orc_ecg_1d(int32_t n, const double *v, double dx, double x0);

/* ---- grids (2D/3D): GPU3D.cu:1487-1680, new_11.cu:1535-1689, 352-417 ---- */

/* Mirror-boundary map.  grid: nx*ny*nz cell types (LQT_EMPTY = not tissue).
 * Out: tissue_of[nx*ny*nz] = tissue index (>=0), or -(k+1) for a boundary
 * voxel mirrored to tissue k, or INT32_MIN for other empty voxels.  Tissue
 * voxels are numbered x-major (GPU3D.cu:1307-1333).  Returns tissue count. */
int64_t orc_build_map(int32_t nx, int32_t ny, int32_t nz, const uint8_t *grid,
                      int32_t *tissue_of);

/* Per-tissue diffusion tensor and its divergence.  d6: [ntissue][6] =
 * D_xx, D_yy, D_zz, D_xy, D_xz, D_yz with D = d_t I + (d_f - d_t) f f^T;
 * b3: [ntissue][3] = sum_i dD_ij/dx_i by central differences between tissue
 * neighbours, one-sided next to non-tissue (new_11.cu:383-408). */
void orc_build_tensor(int32_t nx, int32_t ny, int32_t nz, double dx,
                      const int32_t *tissue_of, const int64_t *tissue_cell,
                      int64_t ntissue, const float *fibre, double d_f,
                      double d_t, double *d6, double *b3);

/* One forward-Euler diffusion + TPORd step of every tissue voxel.
 * v_grid values come from the current state; istim: per tissue voxel. */
void orc_grid_step(int32_t nx, int32_t ny, int32_t nz, double dx,
                   const int32_t *tissue_of, const int64_t *tissue_cell,
                   int64_t ntissue, const double *d6, const double *b3,
                   double *state, const uint8_t *ctype, const lqt_model *m,
                   double dt, const double *istim, double *du_out,
                   int nthreads);

/* Pseudo-ECG of a grid (3D form of plot1DECG_compare.py:89-105). */
double orc_ecg_grid(int32_t nx, int32_t ny, int32_t nz, double dx,
                    const int32_t *tissue_of, const int64_t *tissue_cell,
                    int64_t ntissue, const double *state, const double *r0);

/* Stimulus window test with the reference's floating time
 * (OneD.cc:337-338: time - floor(time/BCL)*BCL in [start, start+dur)). */
int orc_in_window(double time, double bcl, double start, double dur);

#ifdef __cplusplus
}
#endif
#endif
