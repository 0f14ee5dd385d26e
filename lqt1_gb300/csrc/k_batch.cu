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
// cur (or NULL): [n][6] INa, ICaL, IKr, IKs, IK1 and |dV/dt| of the last
// update (getINa / getICaL / getIKr / getIKs / getIK1 / getAbsDvdt,
// SingleCell/TPORd.cc:358-376).
template <typename R>
__global__ void __launch_bounds__(128) k_cells_update(SoA<R> s, const uint8_t *__restrict__ ctype,
                                                      const double *__restrict__ ist,
                                                      const double *__restrict__ dvgap, double *__restrict__ dvdt,
                                                      double *__restrict__ cur, const ModelK *__restrict__ models,
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
        if (cur) {
            double *ci = cur + 6 * i;
            ci[0] = (double)o.ina;
            ci[1] = (double)o.ical;
            ci[2] = (double)o.ikr;
            ci[3] = (double)o.iks;
            ci[4] = (double)o.ik1;
            ci[5] = fabs((double)o.dvdt);
        }
    }
}

// ------------------------------------------------------------------------
// Persistent batch kernel.  MAXT = CTA width (cells per item), MINB = minimum
// resident CTAs per SM the register allocation must allow (the autotuner in
// api_batch.cu picks the pair).
template <typename R, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_batch(BatchDev<R> b, StepT<R> k)
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
        R vmax = (R)-100;    // the starting value of maxEndo / maxEpi, OneD_VW.cc:246-247
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

        const int64_t nsteps_item = b.step_cap > 0 && b.step_cap < item.nsteps ? b.step_cap : item.nsteps;
        const int64_t nsteps_seg = b.step_cap > 0 && b.step_cap < seg.nsteps ? b.step_cap : seg.nsteps;
        for (int64_t st = 0; st < nsteps_item; ++st) {
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
            if (active && st < nsteps_seg) {
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
                const bool s1_open = st >= w_on && st < w_off;
                const bool on = s1_open && li < seg.n_stim;
                // S2 only while no S1 window is open (OneD_VW.cc:265-279)
                const bool on2 = !s1_open && st >= seg.s2_on && st < seg.s2_off && li >= seg.s2_c0 &&
                                 li < seg.s2_c0 + seg.s2_n;
                const R ist = on ? stim : (on2 ? (R)seg.s2_stim : (R)0);
                if (opened && b.det_t_act) {
                    det_open_cycle(det, (float)vo);
                    ++beat;
                }
                StepOut<R> o{};
                tpord_step<R>(c, ct, m, k, ist, dvgap, &o);
                vbuf[cur ^ 1][t] = c.v;
                if (st >= seg.vmax_from && c.v >= vmax) vmax = c.v;

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
                        b.rec_v[((int64_t)seg.rec_slot * b.rec_cap + slot) * b.rec_width + li] = (double)c.v;
                        if (li == 0) b.rec_t[(int64_t)seg.rec_slot * b.rec_cap + slot] = time;
                        if (li == 0 && seg.rec_cur) {
                            double *rc = b.rec_cur + ((int64_t)seg.rec_slot * b.rec_cap + slot) * 2;
                            rc[0] = (double)o.ical;
                            rc[1] = (double)o.iks;
                        }
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
        if (item.ecg_seg >= 0 && nsteps_item > 0 && ((nsteps_item - 1) % b.rec_every) == 0) {
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
                const int64_t slot = (nsteps_item - 1) / b.rec_every;
                if (slot < b.rec_cap) b.ecg[(int64_t)b.segs[item.ecg_seg].rec_slot * b.rec_cap + slot] = acc;
            }
        }
        if (active) {
            store_cell(c, b.s, cell);
            b.s.v[cell] = c.v;
            if (b.det_beats) b.det_beats[cell] = nact;
            if (b.vmax) b.vmax[cell] = (float)vmax;
        }
    }
}

// ---- host-side launchers -------------------------------------------------
template <typename R>
cudaError_t launch_cells_update(const SoA<R> &s, const uint8_t *ctype, const double *ist, const double *dvgap,
                                double *dvdt, double *cur, const ModelK *models, const uint16_t *model_of,
                                const StepK &k, int64_t n, int64_t nsteps, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int bs = 128;
    int64_t nb = (n + bs - 1) / bs;
    if (nb > 152 * 64) nb = 152 * 64;
    k_cells_update<R><<<(unsigned)nb, bs, 0, stream>>>(s, ctype, ist, dvgap, dvdt, cur, models, model_of,
                                                       step_as<R>(k), n, nsteps);
    return cudaGetLastError();
}

// (width, minimum CTAs/SM) variants compiled for each precision
#define LQT_BATCH_VARIANTS_F32(X) X(float, 128, 4) X(float, 128, 6) X(float, 256, 2) X(float, 256, 3) X(float, 512, 1)
#define LQT_BATCH_VARIANTS_F64(X) X(double, 128, 1) X(double, 256, 1) X(double, 512, 1)

template <typename R>
cudaError_t launch_batch(const BatchDev<R> &b, const StepK &k, int threads, int minb, int ctas, cudaStream_t stream)
{
    if (b.nitems <= 0) return cudaSuccess;
    const StepT<R> kk = step_as<R>(k);
#define LQT_LAUNCH(RR, T, M)                                                                   \
    if (sizeof(R) == sizeof(RR) && threads == T && minb == M) {                                \
        k_batch<R, T, M><<<ctas, T, 0, stream>>>(b, kk);                                       \
        return cudaGetLastError();                                                             \
    }
    if constexpr (sizeof(R) == 4) {
        LQT_BATCH_VARIANTS_F32(LQT_LAUNCH)
    } else {
        LQT_BATCH_VARIANTS_F64(LQT_LAUNCH)
    }
#undef LQT_LAUNCH
    return cudaErrorInvalidConfiguration;
}

template cudaError_t launch_cells_update<double>(const SoA<double> &, const uint8_t *, const double *,
                                                 const double *, double *, double *, const ModelK *,
                                                 const uint16_t *, const StepK &, int64_t, int64_t, cudaStream_t);
template cudaError_t launch_cells_update<float>(const SoA<float> &, const uint8_t *, const double *, const double *,
                                                double *, double *, const ModelK *, const uint16_t *, const StepK &,
                                                int64_t, int64_t, cudaStream_t);
template cudaError_t launch_batch<double>(const BatchDev<double> &, const StepK &, int, int, int, cudaStream_t);
template cudaError_t launch_batch<float>(const BatchDev<float> &, const StepK &, int, int, int, cudaStream_t);

}  // namespace lqt

namespace lqt {
// Resident CTAs per SM of a variant, and the variant list (autotuner input).
template <typename R> int batch_max_ctas_per_sm(int threads, int minb)
{
    int n = 0;
    cudaError_t e = cudaErrorInvalidConfiguration;
#define LQT_OCC(RR, T, M)                                                                      \
    if (sizeof(R) == sizeof(RR) && threads == T && minb == M)                                  \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<R, T, M>, T, 0);
    if constexpr (sizeof(R) == 4) {
        LQT_BATCH_VARIANTS_F32(LQT_OCC)
    } else {
        LQT_BATCH_VARIANTS_F64(LQT_OCC)
    }
#undef LQT_OCC
    return e == cudaSuccess ? n : 0;
}
template int batch_max_ctas_per_sm<double>(int, int);
template int batch_max_ctas_per_sm<float>(int, int);

template <typename R> std::vector<std::pair<int, int>> batch_variants()
{
    std::vector<std::pair<int, int>> v;
#define LQT_LIST(RR, T, M) v.emplace_back(T, M);
    if constexpr (sizeof(R) == 4) {
        LQT_BATCH_VARIANTS_F32(LQT_LIST)
    } else {
        LQT_BATCH_VARIANTS_F64(LQT_LIST)
    }
#undef LQT_LIST
    return v;
}
template std::vector<std::pair<int, int>> batch_variants<double>();
template std::vector<std::pair<int, int>> batch_variants<float>();
}  // namespace lqt
