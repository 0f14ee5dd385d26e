// k_batch.cu -- persistent kernel for batches of independent instances
// (single cells and 1D strands) and the Cell-interface update kernel.
//
// Replaces the reference's per-cell CPU loops: OneD.cc:317-398 (strand:
// stimulus, mirrored-end diffusion, update) and SingleCell.cc:95-109 (single
// cell), for thousands of uneven instances in one launch.
//
// Work decomposition: the host groups instances into items whose cells are a
// contiguous range of at most blockDim cells (one strand, or a pack of single
// cells / short strands with similar step counts).  Each CTA pulls items from
// an atomic queue (largest first) and runs every step of the item with the
// state in registers and V exchanged through shared memory, so HBM is touched
// only to load/store state once per item and to write outputs.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "api_common.h"
#include "lqt_internal.h"

namespace lqt {

// ------------------------------------------------------------------------
// Cell interface: n independent cells, nsteps updates with fixed inputs
// (TPORd::setIstim / setDVgap_dt / update, SingleCell/TPORd.cc:358-379).
template <typename R>
__global__ void __launch_bounds__(128) k_cells_update(SoA<R> s, const uint8_t *__restrict__ ctype,
                                                      const double *__restrict__ ist,
                                                      const double *__restrict__ dvgap, double *__restrict__ dvdt,
                                                      const ModelK *__restrict__ models,
                                                      const uint16_t *__restrict__ model_of, StepT<R> k, int64_t n,
                                                      int64_t nsteps)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        CellState<R> c;
        load_cell(c, s, i);
        c.v = s.v[i];
        const ModelT<R> m = model_as<R>(models[model_of ? model_of[i] : 0]);
        const R is = ist ? (R)ist[i] : (R)0;
        const R dg = dvgap ? (R)dvgap[i] : (R)0;
        const int ct = ctype[i];
        StepOut<R> o{};
        for (int64_t t = 0; t < nsteps; ++t) tpord_step<R>(c, ct, m, k, is, dg, &o);
        store_cell(c, s, i);
        s.v[i] = c.v;
        if (dvdt) dvdt[i] = (double)o.dvdt;
    }
}

// ------------------------------------------------------------------------
// Persistent batch kernel.
template <typename R, int MAXT>
__global__ void __launch_bounds__(MAXT) k_batch(BatchDev<R> b, StepT<R> k)
{
    __shared__ R vbuf[2][MAXT];
    __shared__ double red[MAXT / 32];
    __shared__ int s_item;

    const int t = threadIdx.x;
    for (;;) {
        __syncthreads();
        if (t == 0) s_item = atomicAdd(b.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= b.nitems) break;
        const Item item = b.items[it];
        const bool active = t < item.ncells;
        const int64_t cell = item.cell0 + t;

        // per-thread segment data
        Seg seg{};
        int li = 0;
        CellState<R> c{};
        int ct = 3;
        R coeff = 0, dcoeff = 0;
        ModelT<R> m{};
        if (active) {
            seg = b.segs[b.seg_of[cell]];
            li = (int)(cell - seg.cell0);
            load_cell(c, b.s, cell);
            c.v = b.s.v[cell];
            ct = b.ctype[cell];
            coeff = b.coeff ? (R)b.coeff[cell] : (R)0;
            dcoeff = b.dcoeff ? (R)b.dcoeff[cell] : (R)0;
            m = model_as<R>(b.models[seg.model]);
        }
        // stimulus windows: [on, off) step ranges, host-computed from the
        // reference's floating `time += dt` (OneD.cc:317,337-338)
        int wi = 0;
        int64_t w_on = INT64_MAX, w_off = INT64_MAX;
        if (active && seg.nwin > 0) {
            w_on = b.win[seg.win0].on;
            w_off = b.win[seg.win0].off;
        }
        DetState det{};
        det.phase = kDetIdle;
        float t_act = -1.f;
        int beat = 0;        // cycles opened so far
        int nact = 0;        // activations recorded
        const bool strand = seg.n > 1;
        const R dx = (R)seg.dx;
        const R inv_dx = (R)1 / dx, inv_2dx = (R)1 / ((R)2 * dx), inv_dx2 = (R)1 / (dx * dx);
        const R stim = (R)seg.stim;
        double time = 0.0;
        int cur = 0;
        vbuf[0][t] = active ? c.v : (R)0;

        for (int64_t st = 0; st < item.nsteps; ++st) {
            __syncthreads();
            // pseudo-ECG of the previous recorded step (needs all V of that step)
            if (item.ecg_seg >= 0 && st > 0 && ((st - 1) % b.rec_every) == 0) {
                double term = 0.0;
                if (active) {
                    const R *V = vbuf[cur];
                    const double r = li * (double)seg.dx - seg.ecg_x0;
                    double dv;
                    if (li == 0) dv = (double)V[t + 1] - (double)V[t];
                    else if (li == seg.n - 1) dv = (double)V[t] - (double)V[t - 1];
                    else dv = 0.5 * ((double)V[t + 1] - (double)V[t - 1]);
                    term = -dv / (r * r);
                }
                for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
                if ((t & 31) == 0) red[t >> 5] = term;
                __syncthreads();
                if (t == 0) {
                    double acc = 0.0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) acc += red[w];
                    const int64_t slot = (st - 1) / b.rec_every;
                    if (slot < b.rec_cap) b.ecg[(int64_t)b.segs[item.ecg_seg].rec_slot * b.rec_cap + slot] = acc;
                }
            }
            if (active && st < seg.nsteps) {
                const R *V = vbuf[cur];
                const R vo = V[t];
                // diffusion, OneD.cc:366-391 (mirrored ends)
                R dvgap = 0;
                if (strand) {
                    R fo, so;
                    if (li == 0) {
                        fo = (V[t + 1] - vo) * inv_dx;
                        so = (V[t + 1] + vo - (R)2 * vo) * inv_dx2;
                    } else if (li == seg.n - 1) {
                        fo = (vo - V[t - 1]) * inv_dx;
                        so = (vo + V[t - 1] - (R)2 * vo) * inv_dx2;
                    } else {
                        fo = (V[t + 1] - V[t - 1]) * inv_2dx;
                        so = (V[t + 1] + V[t - 1] - (R)2 * vo) * inv_dx2;
                    }
                    dvgap = dcoeff * fo + coeff * so;
                }
                // stimulus
                bool opened = false;
                if (st >= w_off) {
                    ++wi;
                    if (wi < seg.nwin) {
                        w_on = b.win[seg.win0 + wi].on;
                        w_off = b.win[seg.win0 + wi].off;
                    } else {
                        w_on = w_off = INT64_MAX;
                    }
                }
                if (st == w_on) opened = true;
                const bool on = st >= w_on && st < w_off && li < seg.n_stim;
                const R ist = on ? stim : (R)0;
                if (opened && b.det_t_act) {
                    det_open_cycle(det, (float)vo);
                    ++beat;
                }
                StepOut<R> o{};
                tpord_step<R>(c, ct, m, k, ist, dvgap, &o);
                vbuf[cur ^ 1][t] = c.v;

                if (b.det_t_act && det.phase != kDetIdle) {
                    DetEvent ev;
                    if (det_step(det, (float)vo, (float)c.v, (float)o.dvdt, (float)time, seg.act_thr, t_act, ev)) {
                        if (ev.t_act >= 0.f && nact < b.max_beats) {
                            b.det_t_act[cell * b.max_beats + nact] = ev.t_act;
                            ++nact;
                        }
                        if (ev.t_90 >= 0.f && nact > 0 && nact - 1 < b.max_beats) {
                            const int64_t o2 = cell * b.max_beats + (nact - 1);
                            b.det_apd90[o2] = ev.apd90;
                            b.det_dvdt[o2] = ev.dvdt_max;
                            if (ev.ead) b.det_ead[cell] = 1;
                        }
                    }
                }
                if (seg.rec_slot >= 0 && (st % b.rec_every) == 0) {
                    const int64_t slot = st / b.rec_every;
                    if (slot < b.rec_cap) {
                        b.rec_v[((int64_t)seg.rec_slot * b.rec_cap + slot) * b.rec_width + li] = (float)c.v;
                        if (li == 0) b.rec_t[(int64_t)seg.rec_slot * b.rec_cap + slot] = time;
                    }
                }
                if (!(c.v == c.v) || c.v < (R)b.vmin_ok || c.v > (R)b.vmax_ok) atomicAdd(b.nbad, 1ull);
            } else if (active) {
                vbuf[cur ^ 1][t] = vbuf[cur][t];
            }
            time += b.dt;
            cur ^= 1;
        }
        // ECG of the final recorded step
        __syncthreads();
        if (item.ecg_seg >= 0 && item.nsteps > 0 && ((item.nsteps - 1) % b.rec_every) == 0) {
            double term = 0.0;
            if (active) {
                const R *V = vbuf[cur];
                const double r = li * (double)seg.dx - seg.ecg_x0;
                double dv;
                if (li == 0) dv = (double)V[t + 1] - (double)V[t];
                else if (li == seg.n - 1) dv = (double)V[t] - (double)V[t - 1];
                else dv = 0.5 * ((double)V[t + 1] - (double)V[t - 1]);
                term = -dv / (r * r);
            }
            for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
            if ((t & 31) == 0) red[t >> 5] = term;
            __syncthreads();
            if (t == 0) {
                double acc = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) acc += red[w];
                const int64_t slot = (item.nsteps - 1) / b.rec_every;
                if (slot < b.rec_cap) b.ecg[(int64_t)b.segs[item.ecg_seg].rec_slot * b.rec_cap + slot] = acc;
            }
        }
        if (active) {
            store_cell(c, b.s, cell);
            b.s.v[cell] = c.v;
            if (b.det_beats) b.det_beats[cell] = nact;
        }
    }
}

// ---- host-side launchers -------------------------------------------------
template <typename R>
cudaError_t launch_cells_update(const SoA<R> &s, const uint8_t *ctype, const double *ist, const double *dvgap,
                                double *dvdt, const ModelK *models, const uint16_t *model_of, const StepK &k,
                                int64_t n, int64_t nsteps, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int bs = 128;
    int64_t nb = (n + bs - 1) / bs;
    if (nb > 152 * 64) nb = 152 * 64;
    k_cells_update<R><<<(unsigned)nb, bs, 0, stream>>>(s, ctype, ist, dvgap, dvdt, models, model_of, step_as<R>(k), n,
                                                       nsteps);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_batch(const BatchDev<R> &b, const StepK &k, int threads, int ctas, cudaStream_t stream)
{
    if (b.nitems <= 0) return cudaSuccess;
    if (threads <= 128)
        k_batch<R, 128><<<ctas, 128, 0, stream>>>(b, step_as<R>(k));
    else if (threads <= 256)
        k_batch<R, 256><<<ctas, 256, 0, stream>>>(b, step_as<R>(k));
    else
        k_batch<R, 512><<<ctas, 512, 0, stream>>>(b, step_as<R>(k));
    return cudaGetLastError();
}

template cudaError_t launch_cells_update<double>(const SoA<double> &, const uint8_t *, const double *,
                                                 const double *, double *, const ModelK *, const uint16_t *,
                                                 const StepK &, int64_t, int64_t, cudaStream_t);
template cudaError_t launch_cells_update<float>(const SoA<float> &, const uint8_t *, const double *, const double *,
                                                double *, const ModelK *, const uint16_t *, const StepK &, int64_t,
                                                int64_t, cudaStream_t);
template cudaError_t launch_batch<double>(const BatchDev<double> &, const StepK &, int, int, cudaStream_t);
template cudaError_t launch_batch<float>(const BatchDev<float> &, const StepK &, int, int, cudaStream_t);

}  // namespace lqt

namespace lqt {
// Resident CTAs per SM for the batch kernel at a given width (autotuner input).
template <typename R> int batch_max_ctas_per_sm(int threads)
{
    int n = 0;
    cudaError_t e;
    if (threads <= 128)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<R, 128>, 128, 0);
    else if (threads <= 256)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<R, 256>, 256, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<R, 512>, 512, 0);
    return e == cudaSuccess ? n : 1;
}
template int batch_max_ctas_per_sm<double>(int);
template int batch_max_ctas_per_sm<float>(int);
}  // namespace lqt
