// grid_dev.h -- device view of a tissue grid simulation (k_grid.cuh, api_sim.cu).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lqt_internal.h"

namespace lqt {

constexpr uint8_t kCtlType = 7;    // bits 0-2: LQT_* cell type (0..4)
constexpr uint8_t kCtlS1 = 8;      // receives S1
constexpr uint8_t kCtlS2 = 16;     // receives S2
constexpr int kMaxElectrodes = 8;

// Per-step control, advanced on the device by k_ghost so that a run of steps
// can be captured in one CUDA graph.
struct Clock {
    int64_t step;
    double time;        // accumulated as `time += dt` (OneD.cc:317)
    float time_f;       // the same, rounded once for the detectors
    double tb;          // time - floor(time/bcl)*bcl (only kept with onsets)
    int32_t widx;       // current S1 window
    int32_t s1_on, s2_on, opened, s1_cycle_ok, pad;
};

template <typename R> struct GridDev {
    SoA<R> s;                      // per tissue voxel
    R *vg[2];                      // dense V grids (1D: tissue order)
    const int32_t *gidx;           // tissue -> dense index
    const uint8_t *ctl;            // type + stimulus bits
    const R *d6, *b3;              // anisotropic tensor and its divergence, or null
    const R *coeff, *dcoeff;       // 1D: D and dD/dx per cell
    R diso;                        // isotropic D
    int64_t ntissue, nbnd;
    int64_t sx, sy;                // dense strides of x and y (z stride 1)
    int64_t pad;                   // grid origin offset (0)
    double dx;
    R inv_dx, inv_2dx, inv_dx2, inv_4dx2;
    // 2D/3D: (float)(i * dx) for i < max(nx, ny, nz), the voxel coordinates
    // in mm that the pseudo-ECG uses (rounded once from FP64 on the host)
    const float *xpos;
    double dt;
    ModelT<R> model;
    Clock *clk;
    const Win *win;                // S1 windows
    int32_t nwin;
    int32_t s1_beats;
    Win s2_win;
    double bcl, s1_start, s1_dur;
    R s1_strength, s2_strength;
    const float *onset;            // per tissue voxel onset delay, or null
    const int32_t *bnd_dst, *bnd_src;
    float4 *det;                   // {vrest, vpeak, t_act, bits}, or null
    float *apd90;
    float act_thr;
    R vmin_ok, vmax_ok;
    unsigned long long *nbad;
    // learned surrogate (mixed form): per tissue voxel, the ionic dV/dt fixed
    // for the current macro step, or NaN where the plain step runs; and the
    // list of the voxels that run the plain step (plist_n entries); null = off
    const float *srate;
    const uint8_t *sdflag;         // 1 = the voxel's detector runs during the macro step
    const int32_t *plist;
    const int64_t *plist_n;
    int *serr;                     // bit 1 set when a substep's copy wait ran out
    // the tensor rows that the surrogate's V-only substep streams, in FP16, 3
    // half2 per voxel: (g_x g_y | g_z b_x | b_y b_z), with the tensor
    // D = sub_dtr I + sub_dsg g g^T (g = sqrt|D_f - D_t| times the fibre
    // direction, sub_dsg its sign) and b its divergence; null without a
    // surrogate or on isotropic grids
    const __half2 *t3h;
    float sub_dtr, sub_dsg;
    // test of the failure path (lqt_sim_set_wait_test): 1 = the staged
    // substep leaves out the first tile's copies of every CTA, so that wait
    // runs out; wait_limit = polls per wait (0 = the default limit)
    int32_t sub_skip_copy;
    uint32_t sub_wait_limit;
    // V-halo staging of the 3D substep (variants 200 + CTAs/SM): per tile of
    // kSubTile voxels the box of the dense V grid its 19-point stencils reach,
    // as whole z-segments of its columns; vbox_hdr[8 per tile] = {ok, zlo,
    // xlo, ylo, bx, by, bz, 0} (ok = 0: the box is larger than the stage, the
    // tile reads V from the grid); vli[k] = the voxel's index in its box,
    // ((x - xlo) * by + (y - ylo)) * bz + (z - zlo).  Null = not built.
    const int32_t *vbox_hdr;
    const int32_t *vli;
};

// Floats of a tile's V box in one stage of the staged substep (16 KB), and the
// most columns (z-segment copies) a box may have.
constexpr int kVBoxFloats = 4096;
constexpr int kVBoxMaxCols = 64;

// Voxels per tile of the staged substep kernel; the per-voxel arrays it
// streams (control bytes, dense index, tensor, divergence, rate, detector
// flag) are allocated in whole tiles, so every tile copy is in bounds.
constexpr int kSubTile = 256;
inline int64_t pad_tiles(int64_t n) { return (n + kSubTile - 1) / kSubTile * kSubTile; }

// Occupancy variants of k_grid_step: minimum CTAs/SM of 256 threads.
constexpr int kGridVariantsF32[3] = {2, 3, 4};
constexpr int kGridVariantsF64[2] = {1, 2};

template <typename R>
cudaError_t launch_grid_step(const GridDev<R> &gd, const StepK &k, int cur, int dim, int minb, cudaStream_t st);
template <typename R>
cudaError_t launch_grid_step_minb(const GridDev<R> &gd, const StepT<R> &k, int cur, int dim, int minb, cudaStream_t st);
template <typename R> cudaError_t launch_ghost(const GridDev<R> &gd, int nxt, cudaStream_t st);
// Variants of the V-only substep: minimum CTAs/SM of 256 threads of
// k_sur_substep (5, 6, 8: one thread per voxel, direct loads), of
// k_sur_substep_tile (100 + CTAs/SM: persistent CTAs, each tile's streamed
// rows staged in shared memory by bulk asynchronous copies; 2D/3D
// anisotropic grids, the others fall back to the direct kernel) or of
// k_sur_substep_vbox (200 + CTAs/SM: the same with each tile's V halo box
// staged too; 3D anisotropic grids with nz a multiple of 4 and the boxes
// built, the others fall back to k_sur_substep_tile at 5 CTAs/SM) or of the
// same producer-warp kernel with the rows only (300 + CTAs/SM; 2D/3D
// anisotropic grids, the others fall back as the 100s do).
constexpr int kSubVariants[11] = {5, 6, 8, 105, 106, 108, 203, 204, 304, 305, 306};
constexpr int kSubNVariants = 11;
cudaError_t launch_sur_substep(const GridDev<float> &gd, double dt, int cur, int dim, int minb, cudaStream_t st);
template <typename R>
cudaError_t launch_ecg(const GridDev<R> &gd, int cur, const float4 *el, int nel, double *partial, double *out,
                       double *t_out, int64_t *counter, int64_t cap, int dim, cudaStream_t st);
int64_t ecg_blocks(int64_t ntissue);

}  // namespace lqt
