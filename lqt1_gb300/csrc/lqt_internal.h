// lqt_internal.h -- structures shared by the host API (api.cu) and kernels.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tpord.cuh"

namespace lqt {

constexpr int kNConc = 8;
constexpr int kNGate = 31;

// State of n cells, structure of arrays (layout described in common.cuh).
template <typename R> struct SoA {
    R *v;
    double *conc;
    R *gate;
    int64_t ld;
};

// Stimulus window [on, off) in steps (host-computed, exact w.r.t. the
// reference's floating time accumulation).
struct Win {
    int64_t on, off;
};

// One instance of a batch: a single cell (n == 1) or a strand.
struct Seg {
    int64_t cell0;        // first cell
    int64_t nsteps;       // steps this instance runs
    int32_t n;            // cells
    int32_t n_stim;       // cells [0, n_stim) receive S1 (OneD.cc:340)
    int32_t model;        // index into models[]
    int32_t win0, nwin;   // stimulus windows
    int32_t rec_slot;     // >= 0: V recorded into rec_v[rec_slot]
    double dx;            // mm
    double stim;          // pA/pF
    double ecg_x0;        // electrode position, mm (plot1DECG_compare.py:83)
    float act_thr;        // mV
    int32_t rec_cur;      // 1: ICaL, IKs of the first cell recorded too
    int64_t s2_on, s2_off;  // S2 step range (OneD_VW.cc:273-279)
    int32_t s2_c0, s2_n;    // cells [s2_c0, s2_c0 + s2_n) receive S2
    double s2_stim;         // pA/pF
    int64_t vmax_from;      // first step of the maximum-V watch, INT64_MAX = off
};

// A CTA's unit of work: contiguous cells [cell0, cell0 + ncells).
struct Item {
    int64_t cell0;
    int64_t nsteps;       // max over its segments
    int32_t ncells;
    int32_t ecg_seg;      // segment whose pseudo-ECG is recorded, or -1
};

template <typename R> struct BatchDev {
    SoA<R> s;                        // state
    const uint8_t *ctype;
    const double *coeff, *dcoeff;    // per cell D and dD/dx (OneD.cc:103-131), or null
    const int32_t *seg_of;           // cell -> segment
    const Seg *segs;
    const Item *items;
    int32_t nitems;
    int32_t max_beats;
    const Win *win;
    const ModelK *models;
    double dt;                       // for the FP64 time accumulation (OneD.cc:317)
    int64_t step_cap;                // > 0: stop every item after this many steps (autotuner probes)
    int *queue;                      // atomic work counter
    unsigned long long *nbad;        // blow-up counter
    double vmin_ok, vmax_ok;
    // recording
    int64_t rec_every, rec_cap;
    int32_t rec_width;               // max cells of a recorded segment
    double *rec_v;                   // [slot][rec_cap][rec_width]
    double *rec_cur;                 // [slot][rec_cap][2]: ICaL, IKs of the first cell
    float *vmax;                     // per cell: maximum V since vmax_from, or null
    double *rec_t;                   // [slot][rec_cap]
    double *ecg;                     // [slot][rec_cap]
    // detectors ([cell][max_beats]), or null
    float *det_t_act, *det_apd90, *det_dvdt;
    uint8_t *det_ead;
    int32_t *det_beats;
};

template <typename R>
cudaError_t launch_cells_update(const SoA<R> &s, const uint8_t *ctype, const double *ist, const double *dvgap,
                                double *dvdt, double *cur, const ModelK *models, const uint16_t *model_of,
                                const StepK &k, int64_t n, int64_t nsteps, cudaStream_t stream);
template <typename R>
cudaError_t launch_batch(const BatchDev<R> &b, const StepK &k, int threads, int minb, int ctas, cudaStream_t stream);

// AoS (reference order, double) <-> SoA conversion
template <typename R>
cudaError_t launch_pack(const double *aos, const SoA<R> &s, int64_t n, cudaStream_t st);
template <typename R>
cudaError_t launch_unpack(const SoA<R> &s, double *aos, int64_t n, cudaStream_t st);

}  // namespace lqt

namespace lqt {
template <typename R, typename T>
cudaError_t launch_gather_v(const R *vg, const int32_t *gidx, T *out, int64_t n, cudaStream_t st);
template <typename R> cudaError_t launch_scatter_v(const R *v, const int32_t *gidx, R *vg, int64_t n, cudaStream_t st);
// FP16 tensor rows of the surrogate substep (grid_dev.h, GridDev::t3h) from
// the FP32 tensor and divergence; dtr = D_t, sgn = the sign of D_f - D_t.
cudaError_t launch_tensor_f16(const float *d6, const float *b3, int64_t n, float dtr, float sgn, __half2 *t3h,
                              cudaStream_t st);
template <typename R>
cudaError_t launch_sample_v(const R *vg, const uint8_t *tissue, int32_t nx, int32_t ny, int32_t nz, int32_t stride,
                            int64_t sx, int64_t sy, double *out, cudaStream_t st);
int write_vtk_file(const char *path, const double *samples, int32_t nx, int32_t ny, int32_t nz, int32_t stride);
int64_t vtk_samples(int32_t nx, int32_t ny, int32_t nz, int32_t stride);
}  // namespace lqt
