// api_sim.cu -- lqt_sim_*: 1D/2D/3D tissue simulations on one GPU.
//
// The host loop of the reference (GPU3D.cu:1731-1842, new_11.cu:1755-1890)
// launches five kernels with a device-wide synchronisation between them and
// copies all of V back every step.  Here a step is two kernels (k_grid_step,
// k_ghost) on one stream; runs of steps are captured once into a CUDA graph
// and replayed, the stimulus schedule and time live on the device, the
// blow-up scan is a counter read on request, and the pseudo-ECG is reduced on
// the device every `every` steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "api_common.h"
#include "geometry.h"
#include "grid_dev.h"
#include "sur.h"

using namespace lqt;

namespace {
constexpr int kGraphChunk = 50;   // steps per captured graph (even: V buffer parity is kept;
                                  // a multiple of the surrogate's macro step)
static_assert(kGraphChunk == kSurSpan, "graph chunks must start on macro-step boundaries");
constexpr uint32_t kCkptMagic = 0x4c515443;   // "LQTC"
constexpr uint32_t kCkptVersion = 1;
}  // namespace

struct lqt_sim {
    lqt_sim_params p{};
    int32_t nx = 0, ny = 0, nz = 0, dim = 3;
    double dx = 0.2;
    int64_t ntissue = 0, ngrid = 0, nbnd = 0, ld = 0;
    cudaStream_t stream = nullptr;
    DevMem mem;
    TissueMap tm;
    // device
    void *vg[2] = {nullptr, nullptr};
    void *gate = nullptr, *d6 = nullptr, *b3 = nullptr, *coeff = nullptr, *dcoeff = nullptr;
    __half2 *t3h = nullptr;         // FP16 tensor rows for the surrogate substep (pad_tiles rows)
    double d_fibre = 0, d_trans = 0;  // the anisotropic tensor's coefficients (2D/3D with fibres)
    int32_t *vbox_hdr = nullptr, *vli = nullptr;   // V-halo boxes of the 3D substep (k_sur_substep_vbox)
    double *conc = nullptr, *aos = nullptr;
    int32_t *gidx = nullptr, *bnd_dst = nullptr, *bnd_src = nullptr;
    float *xpos = nullptr;          // 2D/3D: (float)(i * dx), i < max(nx, ny, nz)
    uint8_t *ctl = nullptr;
    float *onset = nullptr;
    Clock *clk = nullptr;
    Win *win = nullptr;
    int64_t win_cap = 0;
    float4 *det = nullptr;
    float *apd90 = nullptr;
    unsigned long long *nbad = nullptr;
    // protocol
    bool has_protocol = false, has_s2 = false;
    bool own_stream = false;
    lqt_protocol proto{};
    std::vector<uint8_t> ctl_host;
    int64_t win_horizon = 0;            // windows valid for steps < win_horizon
    int32_t nwin = 0;
    Win s2win{INT64_MAX, INT64_MAX};
    std::vector<double> times;
    // host mirror of the clock
    int64_t step = 0;
    double time = 0.0;
    int cur = 0;
    // ECG
    int32_t nel = 0, ecg_every = 0;
    float4 *el = nullptr;
    double *ecg_partial = nullptr, *ecg_out = nullptr, *ecg_t = nullptr;
    int64_t *ecg_count = nullptr, ecg_cap = 0;
    // occupancy variant of k_grid_step (minimum CTAs/SM) and the autotuner
    int minb = 2;
    int sub_minb = 5;               // V-only substep variant (kSubVariants)
    bool sub_forced = false;        // set by lqt_sim_substep_variant: the autotuner keeps it
    int32_t sub_skip_copy = 0;      // failure-path test (lqt_sim_set_wait_test)
    uint32_t sub_wait_limit = 0;
    float sub_tune_ms[kSubNVariants] = {};   // last autotune: mean ms per substep variant
    bool tuned = false;
    float tune_ms[4] = {0, 0, 0, 0};
    // learned surrogate (mixed form): network, per-voxel rate, counters
    lqt_mlp *sur = nullptr;
    lqt_sur_config sur_cfg{};
    int sur_nsub = kSurSteps;       // plain steps per macro step
    float *srate = nullptr;
    uint8_t *sdflag = nullptr;
    int32_t *plist = nullptr;
    unsigned long long *plist_n = nullptr;
    bool plist_valid = false;       // rate/list written by a macro-step launch still in effect
    unsigned long long *sur_stats = nullptr;
    int *sur_err = nullptr;
    int64_t sur_launches = 0;
    // asynchronous V read-back: a ring of kVSlots device slots, so that the
    // copies of the short steps between two macro steps can trail behind them
    // and catch up during the long one; each copy is split over kCopyStreams
    // streams (several copy engines share the host link) and joined into one
    // completion event per copy, kept for the last kVDone copies
    static constexpr int kCopyStreams = 4, kVSlots = 16, kVDone = 64;
    void *vslot[kVSlots] = {};
    cudaStream_t copy_stream[kCopyStreams] = {};
    cudaEvent_t gathered = nullptr, chunk_done[kCopyStreams] = {}, vdone[kVDone] = {};
    int64_t v_issued = 0;           // lqt_sim_get_v_async calls so far (the next copy's number)
    // state transfer (lqt_sim_get_state / set_state): the AoS staging buffer
    // (aos) and the tissue-order V, kept after the first use (no allocation
    // or device-wide free per call)
    void *vtmp = nullptr;
    // output sampling: tissue mask of the dense grid, lattice buffer
    uint8_t *tmask = nullptr;
    double *samp = nullptr;
    int64_t samp_cap = 0;
    // graph
    cudaGraphExec_t graph = nullptr;
    int graph_cur = -1;
    bool graph_valid = false;

    ~lqt_sim()
    {
        for (cudaStream_t c : copy_stream)
            if (c) cudaStreamSynchronize(c);
        if (gathered) cudaEventDestroy(gathered);
        for (cudaEvent_t e : chunk_done)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : vdone)
            if (e) cudaEventDestroy(e);
        for (cudaStream_t c : copy_stream)
            if (c) cudaStreamDestroy(c);
        if (graph) cudaGraphExecDestroy(graph);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
    bool fp64() const { return p.precision == LQT_FP64; }

    template <typename R> GridDev<R> dev() const
    {
        GridDev<R> g{};
        g.s = SoA<R>{nullptr, conc, (R *)gate, ld};
        g.vg[0] = (R *)vg[0];
        g.vg[1] = (R *)vg[1];
        g.gidx = gidx;
        g.ctl = ctl;
        g.d6 = (const R *)d6;
        g.b3 = (const R *)b3;
        g.coeff = (const R *)coeff;
        g.dcoeff = (const R *)dcoeff;
        g.ntissue = ntissue;
        g.nbnd = nbnd;
        g.sx = (int64_t)ny * nz;
        g.sy = dim == 2 ? 1 : nz;
        g.pad = 0;
        g.dx = dx;
        g.xpos = xpos;
        g.inv_dx = (R)(1.0 / dx);
        g.inv_2dx = (R)(1.0 / (2.0 * dx));
        g.inv_dx2 = (R)(1.0 / (dx * dx));
        g.inv_4dx2 = (R)(1.0 / (4.0 * dx * dx));
        g.dt = p.dt;
        g.model = model_as<R>(make_modelk(p.model));
        g.clk = clk;
        g.win = win;
        g.nwin = nwin;
        g.s1_beats = proto.s1_beats;
        g.s2_win = s2win;
        g.bcl = has_protocol ? proto.bcl : 1.0;
        g.s1_start = proto.s1_start;
        g.s1_dur = proto.s1_duration;
        g.s1_strength = (R)proto.s1_strength;
        g.s2_strength = (R)proto.s2_strength;
        g.onset = onset;
        g.bnd_dst = bnd_dst;
        g.bnd_src = bnd_src;
        g.det = det;
        g.apd90 = apd90;
        g.act_thr = (float)p.act_threshold;
        g.vmin_ok = (R)p.vmin_ok;
        g.vmax_ok = (R)p.vmax_ok;
        g.nbad = nbad;
        const bool in_macro = sur && plist_valid;
        g.srate = in_macro ? srate : nullptr;
        g.sdflag = in_macro ? sdflag : nullptr;
        g.plist = in_macro ? plist : nullptr;
        g.plist_n = in_macro ? (const int64_t *)plist_n : nullptr;
        g.serr = in_macro ? sur_err : nullptr;
        g.t3h = in_macro ? t3h : nullptr;
        g.sub_dtr = (float)d_trans;
        g.sub_dsg = d_fibre >= d_trans ? 1.f : -1.f;
        g.vbox_hdr = in_macro ? vbox_hdr : nullptr;
        g.vli = in_macro ? vli : nullptr;
        g.sub_skip_copy = sub_skip_copy;
        g.sub_wait_limit = sub_wait_limit;
        return g;
    }
    double diso = 0.154;
};

namespace {

template <typename R> GridDev<R> devf(const lqt_sim *s)
{
    GridDev<R> g = s->dev<R>();
    g.diso = (R)s->diso;
    return g;
}

// V-halo boxes of the 3D substep, per tile of kSubTile tissue voxels (in
// tissue order): the box spans the tile's columns one voxel beyond in x and y
// and its z range one voxel beyond, z rounded out to multiples of 4 and kept
// inside the column (nz is a multiple of 4; tissue is off the grid faces, so
// the box stays inside the grid).  hdr: 8 ints per tile {ok, zlo, xlo, ylo,
// bx, by, bz, 0}, ok = 0 when the box exceeds kVBoxFloats or kVBoxMaxCols
// columns; li: each voxel's index in its tile's box (pad_tiles entries).
void build_vboxes(const std::vector<int64_t> &cells, int64_t nx, int64_t ny, int64_t nz, std::vector<int32_t> &hdr,
                  std::vector<int32_t> &li)
{
    const int64_t n = (int64_t)cells.size(), ntiles = (n + kSubTile - 1) / kSubTile;
    hdr.assign(ntiles * 8, 0);
    li.assign(pad_tiles(n), 0);
    for (int64_t T = 0; T < ntiles; ++T) {
        const int64_t k0 = T * kSubTile, k1 = std::min(n, k0 + kSubTile);
        int64_t xmin = nx, xmax = -1, ymin = ny, ymax = -1, zmin = nz, zmax = -1;
        for (int64_t k = k0; k < k1; ++k) {
            const int64_t g = cells[k], x = g / (ny * nz), y = (g / nz) % ny, z = g % nz;
            xmin = std::min(xmin, x); xmax = std::max(xmax, x);
            ymin = std::min(ymin, y); ymax = std::max(ymax, y);
            zmin = std::min(zmin, z); zmax = std::max(zmax, z);
        }
        const int64_t xlo = xmin - 1, ylo = ymin - 1, zlo = (zmin - 1) / 4 * 4;
        const int64_t bx = xmax + 1 - xlo + 1, by = ymax + 1 - ylo + 1;
        const int64_t bz = std::min(nz - zlo, (zmax + 1 - zlo + 1 + 3) / 4 * 4);
        const bool ok = xlo >= 0 && ylo >= 0 && zmin >= 1 && xmax + 1 < nx && ymax + 1 < ny && zmax + 1 < nz &&
                        bx * by <= kVBoxMaxCols && bx * by * bz <= kVBoxFloats;
        int32_t *h = &hdr[T * 8];
        h[0] = ok;
        h[1] = (int32_t)zlo; h[2] = (int32_t)xlo; h[3] = (int32_t)ylo;
        h[4] = (int32_t)bx; h[5] = (int32_t)by; h[6] = (int32_t)bz;
        if (!ok) continue;
        for (int64_t k = k0; k < k1; ++k) {
            const int64_t g = cells[k], x = g / (ny * nz), y = (g / nz) % ny, z = g % nz;
            li[k] = (int32_t)(((x - xlo) * by + (y - ylo)) * bz + (z - zlo));
        }
    }
}

// Recompute S1 windows for steps [0, horizon) and the S2 window; upload.
int refresh_windows(lqt_sim *s, int64_t horizon)
{
    if (!s->has_protocol) {
        s->nwin = 0;
        s->win_horizon = INT64_MAX;
        return LQT_OK;
    }
    const lqt_protocol &q = s->proto;
    const double t_end = horizon * s->p.dt + 10 * s->p.dt;
    time_axis(s->p.dt, t_end, s->times);
    const int64_t ns = std::min<int64_t>((int64_t)s->times.size(), horizon + 8);
    std::vector<Win> w;
    if (!s->onset) stim_windows(s->times, ns, s->p.dt, q.bcl, q.s1_start, q.s1_duration, q.s1_beats, w);
    if ((int64_t)w.size() > s->win_cap) {
        int64_t cap = std::max<int64_t>(64, (int64_t)w.size() * 2);
        Win *nw = nullptr;
        if (s->mem.alloc((void **)&nw, cap * sizeof(Win))) return LQT_ERR_NOMEM;
        s->win = nw;
        s->win_cap = cap;
        s->graph_valid = false;
    }
    if (!w.empty()) CK(cudaMemcpyAsync(s->win, w.data(), w.size() * sizeof(Win), cudaMemcpyHostToDevice, s->stream));
    if ((int32_t)w.size() != s->nwin) s->graph_valid = false;
    s->nwin = (int32_t)w.size();
    // S2: steps whose time is in [s2_time, s2_time + s2_duration)
    Win s2{INT64_MAX, INT64_MAX};
    if (s->has_s2 && q.s2_time >= 0 && q.s2_duration > 0) {
        for (int64_t k = 0; k < ns; ++k) {
            const double t = s->times[k];
            const bool in = t >= q.s2_time && t < q.s2_time + q.s2_duration;
            if (in && s2.on == INT64_MAX) s2.on = k;
            if (!in && s2.on != INT64_MAX) {
                s2.off = k;
                break;
            }
        }
        if (s2.on != INT64_MAX && s2.off == INT64_MAX) s2.off = ns;
    }
    if (s2.on != s->s2win.on || s2.off != s->s2win.off) s->graph_valid = false;
    s->s2win = s2;
    s->win_horizon = ns - 8;
    // the device clock for the current step
    Clock c{};
    c.step = s->step;
    c.time = s->time;
    c.time_f = (float)s->time;
    int32_t wi = 0;
    while (wi < s->nwin && s->step >= w[wi].off) ++wi;
    c.widx = wi;
    c.s1_on = wi < s->nwin && s->step >= w[wi].on;
    c.opened = wi < s->nwin && s->step == w[wi].on;
    c.s2_on = s->step >= s2.on && s->step < s2.off;
    c.tb = s->time - std::floor(s->time / q.bcl) * q.bcl;
    c.s1_cycle_ok = q.s1_beats <= 0 || std::floor(s->time / q.bcl) < q.s1_beats;
    CK(cudaMemcpyAsync(s->clk, &c, sizeof(c), cudaMemcpyHostToDevice, s->stream));
    return LQT_OK;
}

// At a macro-step boundary with a surrogate attached: the macro-step kernel.
int launch_sur_if_due(lqt_sim *s)
{
    if (!s->sur || s->step % s->sur_nsub != 0) return LQT_OK;
    SurGrid sg{};
    if (!mlp_device_view(s->sur, &sg.w, &sg.norm)) return fail(LQT_ERR_STATE, "surrogate network has no parameters");
    sg.rate = s->srate;
    sg.dflag = s->sdflag;
    sg.plist = s->plist;
    sg.plist_n = s->plist_n;
    sg.stats = s->sur_stats;
    sg.err = s->sur_err;
    sg.kmac = step_as<float>(make_stepk(s->sur_nsub * s->p.dt));
    sg.par[0] = (float)s->p.model.gks_scale;
    sg.par[1] = (float)s->p.model.pca_scale;
    sg.par[2] = (float)s->p.model.gks_iso_scale;
    sg.dvdt_max = (float)s->sur_cfg.dvdt_max;
    sg.foot_dvdt = s->sur_cfg.foot_dvdt > 0 ? (float)s->sur_cfg.foot_dvdt : INFINITY;
    sg.foot_v = (float)s->sur_cfg.foot_v;
    sg.kappa = (float)s->sur_cfg.kappa;
    sg.vstep_max = (float)s->sur_cfg.vstep_max;
    sg.nsub = s->sur_nsub;
    sg.inv_dt = (float)(1.0 / s->p.dt);
    sg.inv_mac = (float)(1.0 / (s->sur_nsub * s->p.dt));
    sg.use_net = s->sur_cfg.use_net;
    CK(cudaMemsetAsync(s->plist_n, 0, sizeof(unsigned long long), s->stream));
    CK(launch_sur_grid(devf<float>(s), sg, s->cur, s->dim, s->stream));
    s->sur_launches += 1;
    s->plist_valid = true;
    return LQT_OK;
}

// The step kernels of one step (without the ghost refresh): the fused plain
// step over all voxels, or, inside a surrogate macro step, the V-only step of
// the surrogate voxels and the plain step over the listed ones.
cudaError_t launch_substep(lqt_sim *s)
{
    const StepK k = make_stepk(s->p.dt);
    if (s->fp64()) return launch_grid_step<double>(devf<double>(s), k, s->cur, s->dim, s->minb, s->stream);
    const GridDev<float> g = devf<float>(s);
    if (g.srate) {
        cudaError_t e = launch_sur_substep(g, s->p.dt, s->cur, s->dim, s->sub_minb, s->stream);
        if (e != cudaSuccess) return e;
    }
    return launch_grid_step<float>(g, k, s->cur, s->dim, s->minb, s->stream);
}

cudaError_t launch_ghost_now(lqt_sim *s)
{
    return s->fp64() ? launch_ghost<double>(devf<double>(s), s->cur ^ 1, s->stream)
                     : launch_ghost<float>(devf<float>(s), s->cur ^ 1, s->stream);
}

int launch_step(lqt_sim *s)
{
    int rc = launch_sur_if_due(s);
    if (rc) return rc;
    CK(launch_substep(s));
    CK(launch_ghost_now(s));
    s->cur ^= 1;
    return LQT_OK;
}

int launch_ecg_now(lqt_sim *s)
{
    if (s->fp64())
        CK(launch_ecg<double>(devf<double>(s), s->cur, s->el, s->nel, s->ecg_partial, s->ecg_out, s->ecg_t,
                              s->ecg_count, s->ecg_cap, s->dim, s->stream));
    else
        CK(launch_ecg<float>(devf<float>(s), s->cur, s->el, s->nel, s->ecg_partial, s->ecg_out, s->ecg_t,
                             s->ecg_count, s->ecg_cap, s->dim, s->stream));
    return LQT_OK;
}

// One step plus, when due, an ECG sample of the new V.
int step_once(lqt_sim *s)
{
    int rc = launch_step(s);
    if (rc) return rc;
    s->step += 1;
    s->time += s->p.dt;
    if (s->nel > 0 && s->ecg_every > 0 && s->step % s->ecg_every == 0) return launch_ecg_now(s);
    return LQT_OK;
}

// Autotuner: time `per` real steps with each occupancy variant of the step
// kernels (CUDA events around the step kernels only) and keep the fastest.
// The variants take turns step by step, so each sees the same phases of the
// simulation (with a surrogate attached, the share of plain voxels changes
// from one macro step to the next); the first round only loads the modules.
// The variants differ only in register allocation, so the steps are valid
// simulation steps whichever variant runs them.  Returns the steps consumed.
int autotune(lqt_sim *s, int per, int64_t *consumed)
{
    const int *cand = s->fp64() ? kGridVariantsF64 : kGridVariantsF32;
    const int ncand = s->dim == 1 ? 1 : (s->fp64() ? 2 : 3);
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    float tot[4] = {0, 0, 0, 0};
    int rc = LQT_OK;
    *consumed = 0;
    for (int i = 0; i < per && rc == LQT_OK; ++i) {
        for (int c = 0; c < ncand && rc == LQT_OK; ++c) {
            s->minb = cand[c];
            rc = launch_sur_if_due(s);
            if (rc) break;
            cudaError_t e = cudaEventRecord(a, s->stream);
            if (e == cudaSuccess) e = launch_substep(s);
            if (e == cudaSuccess) e = cudaEventRecord(b, s->stream);
            if (e == cudaSuccess) e = launch_ghost_now(s);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (e != cudaSuccess) {
                rc = fail(LQT_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
                break;
            }
            s->cur ^= 1;
            s->step += 1;
            s->time += s->p.dt;
            ++*consumed;
            if (s->nel > 0 && s->ecg_every > 0 && s->step % s->ecg_every == 0) rc = launch_ecg_now(s);
            if (i > 0) tot[c] += ms;
        }
    }
    float best = 1e30f;
    int best_m = cand[0];
    for (int c = 0; c < ncand; ++c) {
        const float avg = per > 1 ? tot[c] / (per - 1) : tot[c];
        s->tune_ms[c] = avg;
        if (avg < best) {
            best = avg;
            best_m = cand[c];
        }
    }
    s->minb = best_m;
    // with a surrogate attached: the V-only substep's variant, timed the same
    // way (variants in turn, whole steps, the first round discarded)
    if (rc == LQT_OK && s->sur && !s->fp64() && !s->sub_forced) {
        float ts[kSubNVariants] = {};
        for (int i = 0; i < per && rc == LQT_OK; ++i) {
            for (int c = 0; c < kSubNVariants && rc == LQT_OK; ++c) {
                s->sub_minb = kSubVariants[c];
                rc = launch_sur_if_due(s);
                if (rc) break;
                const GridDev<float> g = devf<float>(s);
                cudaError_t e = cudaEventRecord(a, s->stream);
                if (e == cudaSuccess && g.srate) e = launch_sur_substep(g, s->p.dt, s->cur, s->dim, s->sub_minb, s->stream);
                if (e == cudaSuccess) e = cudaEventRecord(b, s->stream);
                if (e == cudaSuccess) e = launch_grid_step<float>(g, make_stepk(s->p.dt), s->cur, s->dim, s->minb, s->stream);
                if (e == cudaSuccess) e = launch_ghost_now(s);
                if (e == cudaSuccess) e = cudaEventSynchronize(b);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
                if (e != cudaSuccess) {
                    rc = fail(LQT_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
                    break;
                }
                s->cur ^= 1;
                s->step += 1;
                s->time += s->p.dt;
                ++*consumed;
                if (s->nel > 0 && s->ecg_every > 0 && s->step % s->ecg_every == 0) rc = launch_ecg_now(s);
                if (i > 0) ts[c] += ms;
            }
        }
        int bs = 0;
        for (int c = 1; c < kSubNVariants; ++c)
            if (ts[c] < ts[bs]) bs = c;
        for (int c = 0; c < kSubNVariants; ++c) s->sub_tune_ms[c] = per > 1 ? ts[c] / (per - 1) : ts[c];
        s->sub_minb = kSubVariants[bs];
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    s->tuned = true;
    s->graph_valid = false;
    return rc;
}

// 1 where a dense-grid voxel is tissue (uploaded on first use).
int ensure_tmask(lqt_sim *s)
{
    if (s->tmask) return LQT_OK;
    std::vector<uint8_t> m((size_t)s->ngrid, 0);
    for (int64_t k = 0; k < s->ntissue; ++k) m[(size_t)s->tm.cells[k]] = 1;
    if (s->mem.alloc((void **)&s->tmask, s->ngrid)) return LQT_ERR_NOMEM;
    CK(cudaMemcpy(s->tmask, m.data(), s->ngrid, cudaMemcpyHostToDevice));
    return LQT_OK;
}

// The VTK lattice of the current V into dev_out (device), on the simulation's stream.
int sample_launch(lqt_sim *s, int32_t stride, double *dev_out)
{
    int rc = ensure_tmask(s);
    if (rc) return rc;
    const int64_t sx = (int64_t)s->ny * s->nz, sy = s->dim == 2 ? 1 : s->nz;
    if (s->fp64())
        CK(launch_sample_v<double>((const double *)s->vg[s->cur], s->tmask, s->nx, s->ny, s->nz, stride, sx, sy,
                                   dev_out, s->stream));
    else
        CK(launch_sample_v<float>((const float *)s->vg[s->cur], s->tmask, s->nx, s->ny, s->nz, stride, sx, sy,
                                  dev_out, s->stream));
    return LQT_OK;
}

int build_graph(lqt_sim *s)
{
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    const int64_t step0 = s->step;
    const double time0 = s->time;
    const int cur0 = s->cur;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = LQT_OK;
    // capture with step numbers aligned to the ECG cadence: the graph is
    // replayed only from steps that are multiples of kGraphChunk
    const int64_t launches0 = s->sur_launches;
    const bool plist0 = s->plist_valid;
    for (int i = 0; i < kGraphChunk && rc == LQT_OK; ++i) rc = step_once(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    s->sur_launches = launches0;
    s->plist_valid = plist0;
    s->step = step0;
    s->time = time0;
    s->cur = cur0;
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    s->graph_valid = true;
    s->graph_cur = cur0;
    return LQT_OK;
}

template <typename R> int upload_conv(lqt_sim *s, void *dst, const std::vector<float> &src)
{
    if (src.empty()) return LQT_OK;
    if (sizeof(R) == 4) {
        CK(cudaMemcpyAsync(dst, src.data(), src.size() * 4, cudaMemcpyHostToDevice, s->stream));
    } else {
        std::vector<double> d(src.begin(), src.end());
        CK(cudaMemcpyAsync(dst, d.data(), d.size() * 8, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return LQT_OK;
}

}  // namespace

extern "C" {

int lqt_sim_create(const lqt_sim_params *params, const lqt_geometry *geom, lqt_sim **out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_sim_create: out is NULL");
    *out = nullptr;
    if (!params || !geom || !geom->cell_type) return fail(LQT_ERR_INVALID, "lqt_sim_create: NULL argument");
    const lqt_sim_params &p = *params;
    if (!(p.dt > 0) || !std::isfinite(p.dt)) return fail(LQT_ERR_INVALID, "lqt_sim_create: dt must be > 0");
    if (p.precision != LQT_FP64 && p.precision != LQT_MIXED) return fail(LQT_ERR_INVALID, "lqt_sim_create: precision");
    int rc = check_model(p.model);
    if (rc) return rc;
    const int32_t nx = geom->nx, ny = geom->ny, nz = geom->nz;
    if (nx < 1 || ny < 1 || nz < 1 || (int64_t)nx * ny * nz > (int64_t)INT32_MAX)
        return fail(LQT_ERR_INVALID, "lqt_sim_create: grid dimensions must be >= 1 and the grid below 2^31 voxels");
    if (!(geom->dx > 0)) return fail(LQT_ERR_INVALID, "lqt_sim_create: dx must be > 0");
    const int dim = (ny == 1 && nz == 1) ? 1 : (nz == 1 ? 2 : 3);
    if (dim == 2 && ny < 3) return fail(LQT_ERR_INVALID, "lqt_sim_create: 2D grids need ny >= 3");
    const int64_t total = (int64_t)nx * ny * nz;
    for (int64_t i = 0; i < total; ++i)
        if (geom->cell_type[i] > LQT_MCELL && geom->cell_type[i] != LQT_EMPTY)
            return fail(LQT_ERR_INVALID, "lqt_sim_create: cell type out of range");
    if (dim == 1) {
        for (int64_t i = 0; i < total; ++i)
            if (geom->cell_type[i] == LQT_EMPTY) return fail(LQT_ERR_INVALID, "lqt_sim_create: 1D strands must be all tissue");
    } else {
        // tissue must not touch the grid faces (the reference warns about it,
        // GPU3D.cu:1287-1289); the stencil reads one voxel beyond tissue
        for (int32_t x = 0; x < nx; ++x)
            for (int32_t y = 0; y < ny; ++y)
                for (int32_t z = 0; z < nz; ++z) {
                    const bool face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 ||
                                      (dim == 3 && (z == 0 || z == nz - 1));
                    if (face && geom->cell_type[((int64_t)x * ny + y) * nz + z] != LQT_EMPTY)
                        return fail(LQT_ERR_INVALID, "lqt_sim_create: tissue on the grid boundary; pad the grid by one empty voxel");
                }
    }
    auto *s = new lqt_sim();
    s->p = p;
    s->minb = p.precision == LQT_FP64 ? 1 : 2;
    s->nx = nx;
    s->ny = ny;
    s->nz = nz;
    s->dim = dim;
    s->dx = geom->dx;
    s->stream = (cudaStream_t)p.stream;
    if (!s->stream) {
        // graph capture needs a stream other than the legacy default stream
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return fail(LQT_ERR_CUDA, "lqt_sim_create: cannot create a stream");
        }
        s->own_stream = true;
    }
    if (!(s->p.vmin_ok < s->p.vmax_ok)) {
        s->p.vmin_ok = -1e30;       // NaN-only check when no range is given
        s->p.vmax_ok = 1e30;
    }
    s->diso = geom->d_fibre;
    s->ngrid = total;
    if (dim == 1) {
        s->tm.cells.resize(nx);
        s->tm.tissue_of.resize(nx);
        for (int32_t i = 0; i < nx; ++i) {
            s->tm.cells[i] = i;
            s->tm.tissue_of[i] = i;
        }
    } else {
        // numbering and mirror-boundary map built on the GPU (k_geom.cu)
        rc = build_tissue_map_gpu(nx, ny, nz, geom->cell_type, s->stream, s->tm);
        if (rc) {
            delete s;
            return rc;
        }
    }
    s->ntissue = (int64_t)s->tm.cells.size();
    s->nbnd = (int64_t)s->tm.bnd_dst.size();
    if (s->ntissue == 0) {
        delete s;
        return fail(LQT_ERR_INVALID, "lqt_sim_create: no tissue voxels");
    }
    s->ld = pad128(s->ntissue);
    const size_t rsz = s->fp64() ? 8 : 4;
    const int64_t n = s->ntissue;
    rc = 0;
    rc |= s->mem.alloc(&s->vg[0], s->ngrid * rsz);
    rc |= s->mem.alloc(&s->vg[1], s->ngrid * rsz);
    rc |= s->mem.alloc(&s->gate, s->ld * rsz * kNGate);
    rc |= s->mem.alloc((void **)&s->conc, s->ld * 8 * kNConc);
    const int64_t npad = pad_tiles(n);     // per-voxel rows the staged substep copies in whole tiles
    rc |= s->mem.alloc((void **)&s->ctl, npad);
    rc |= s->mem.alloc((void **)&s->clk, sizeof(Clock));
    rc |= s->mem.alloc((void **)&s->nbad, sizeof(unsigned long long));
    if (dim > 1) {
        rc |= s->mem.alloc((void **)&s->gidx, npad * 4);
        rc |= s->mem.alloc((void **)&s->bnd_dst, std::max<int64_t>(1, s->nbnd) * 4);
        rc |= s->mem.alloc((void **)&s->bnd_src, std::max<int64_t>(1, s->nbnd) * 4);
    }
    if (dim > 1 && geom->fibre) {
        rc |= s->mem.alloc(&s->d6, npad * 6 * rsz);
        rc |= s->mem.alloc(&s->b3, npad * 3 * rsz);
    }
    if (dim == 1) {
        rc |= s->mem.alloc(&s->coeff, n * rsz);
        rc |= s->mem.alloc(&s->dcoeff, n * rsz);
    }
    if (p.detect) {
        rc |= s->mem.alloc((void **)&s->det, n * sizeof(float4));
        rc |= s->mem.alloc((void **)&s->apd90, n * 4);
    }
    if (rc) {
        std::string m = g_err;
        delete s;
        return fail(LQT_ERR_NOMEM, "lqt_sim_create: " + m);
    }
    cudaStream_t st = s->stream;
    // the device clock is read by k_ghost, which set_state below launches:
    // give it a defined value before any kernel runs
    {
        Clock c0{};
        c0.s1_cycle_ok = 1;
        if (cudaMemcpy(s->clk, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess) {
            delete s;
            return fail(LQT_ERR_CUDA, "lqt_sim_create: clock upload failed");
        }
    }
    // per-voxel control bytes and maps
    s->ctl_host.resize(n);
    for (int64_t k = 0; k < n; ++k) s->ctl_host[k] = geom->cell_type[s->tm.cells[k]] & kCtlType;
    std::vector<int32_t> gi32(dim > 1 ? n : 0), bd(s->nbnd), bs(s->nbnd);
    for (int64_t k = 0; k < (int64_t)gi32.size(); ++k) gi32[k] = (int32_t)s->tm.cells[k];
    for (int64_t j = 0; j < s->nbnd; ++j) {
        bd[j] = (int32_t)s->tm.bnd_dst[j];
        bs[j] = (int32_t)s->tm.bnd_src[j];
    }
    // tile padding past the last voxel: zero (copied, never stepped)
    cudaError_t e = cudaMemsetAsync(s->ctl, 0, npad, st);
    if (e == cudaSuccess && dim > 1) e = cudaMemsetAsync(s->gidx, 0, npad * 4, st);
    if (e == cudaSuccess && s->d6) e = cudaMemsetAsync(s->d6, 0, npad * 6 * rsz, st);
    if (e == cudaSuccess && s->b3) e = cudaMemsetAsync(s->b3, 0, npad * 3 * rsz, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->ctl, s->ctl_host.data(), n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && dim > 1) e = cudaMemcpyAsync(s->gidx, gi32.data(), n * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && s->nbnd) e = cudaMemcpyAsync(s->bnd_dst, bd.data(), s->nbnd * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && s->nbnd) e = cudaMemcpyAsync(s->bnd_src, bs.data(), s->nbnd * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        delete s;
        return fail(LQT_ERR_CUDA, std::string("lqt_sim_create: ") + cudaGetErrorString(e));
    }
    if (!rc && dim > 1) {
        const int32_t nmax = std::max(nx, std::max(ny, nz));
        std::vector<float> xp(nmax);
        for (int32_t i = 0; i < nmax; ++i) xp[i] = (float)(i * geom->dx);
        if (s->mem.alloc((void **)&s->xpos, (size_t)nmax * 4)) rc = LQT_ERR_NOMEM;
        else if (cudaMemcpyAsync(s->xpos, xp.data(), (size_t)nmax * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
                 cudaStreamSynchronize(st) != cudaSuccess)
            rc = fail(LQT_ERR_CUDA, "lqt_sim_create: coordinate table upload failed");
    }
    if (!rc && dim > 1 && geom->fibre) {
        s->d_fibre = geom->d_fibre;
        s->d_trans = geom->d_trans;
        std::vector<float> d6, b3;
        build_tensor(nx, ny, nz, geom->dx, s->tm, geom->fibre, geom->d_fibre, geom->d_trans, d6, b3);
        rc = s->fp64() ? (upload_conv<double>(s, s->d6, d6) | upload_conv<double>(s, s->b3, b3))
                       : (upload_conv<float>(s, s->d6, d6) | upload_conv<float>(s, s->b3, b3));
    }
    if (!rc && dim == 1) {
        // OneD.cc:108-131
        std::vector<float> co(n), dco(n);
        std::vector<double> cd(n);
        for (int64_t i = 0; i < n; ++i) cd[i] = geom->coeff_1d ? geom->coeff_1d[i] : geom->d_fibre;
        std::vector<double> dd(n);
        for (int64_t i = 0; i < n; ++i) {
            if (n == 1) dd[i] = 0;
            else if (i == 0) dd[i] = (cd[i + 1] - cd[i]) / geom->dx;
            else if (i == n - 1) dd[i] = (cd[i] - cd[i - 1]) / geom->dx;
            else dd[i] = (cd[i + 1] - cd[i - 1]) / (2.0 * geom->dx);
        }
        if (s->fp64()) {
            cudaMemcpyAsync(s->coeff, cd.data(), n * 8, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(s->dcoeff, dd.data(), n * 8, cudaMemcpyHostToDevice, st);
        } else {
            for (int64_t i = 0; i < n; ++i) {
                co[i] = (float)cd[i];
                dco[i] = (float)dd[i];
            }
            cudaMemcpyAsync(s->coeff, co.data(), n * 4, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(s->dcoeff, dco.data(), n * 4, cudaMemcpyHostToDevice, st);
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = LQT_ERR_CUDA;
    }
    if (rc) {
        std::string m = g_err;
        delete s;
        return fail(rc, "lqt_sim_create: " + m);
    }
    // initial state everywhere, V0 in both grids (ghosts included)
    std::vector<double> init((size_t)n * 40);
    for (int64_t k = 0; k < n; ++k) initial_state(p.v0, &init[k * 40]);
    rc = lqt_sim_set_state(s, init.data());
    if (!rc) {
        Clock c{};
        c.s1_cycle_ok = 1;
        cudaError_t e2 = cudaMemcpyAsync(s->clk, &c, sizeof(c), cudaMemcpyHostToDevice, st);
        std::vector<float4> d0(s->det ? n : 0, make_float4(0.f, 0.f, -1.f, 0.f));
        if (e2 == cudaSuccess && s->det) e2 = cudaMemcpyAsync(s->det, d0.data(), n * sizeof(float4), cudaMemcpyHostToDevice, st);
        if (e2 == cudaSuccess && s->apd90) e2 = cudaMemsetAsync(s->apd90, 0xff, n * 4, st);
        if (e2 == cudaSuccess) e2 = cudaMemsetAsync(s->nbad, 0, sizeof(unsigned long long), st);
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
        if (e2 != cudaSuccess) rc = fail(LQT_ERR_CUDA, cudaGetErrorString(e2));
    }
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return LQT_OK;
}

void lqt_sim_destroy(lqt_sim *s) { delete s; }

int64_t lqt_sim_num_tissue(const lqt_sim *s) { return s ? s->ntissue : -1; }

int lqt_sim_tissue_index(const lqt_sim *s, int64_t *grid_index_host)
{
    if (!s || !grid_index_host) return fail(LQT_ERR_INVALID, "lqt_sim_tissue_index: NULL");
    std::memcpy(grid_index_host, s->tm.cells.data(), s->ntissue * 8);
    return LQT_OK;
}

double lqt_sim_time(const lqt_sim *s) { return s ? s->time : -1.0; }

int lqt_sim_set_protocol(lqt_sim *s, const lqt_protocol *q)
{
    if (!s || !q) return fail(LQT_ERR_INVALID, "lqt_sim_set_protocol: NULL");
    if (!(q->bcl > 0) || q->s1_duration < 0 || q->s1_beats < 0 || !q->s1_mask)
        return fail(LQT_ERR_INVALID, "lqt_sim_set_protocol: bcl > 0, s1_duration >= 0, s1_beats >= 0, s1_mask required");
    const int64_t n = s->ntissue;
    std::vector<uint8_t> c(s->ctl_host);
    std::vector<float> on;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t g = s->tm.cells[k];
        c[k] = (uint8_t)((c[k] & kCtlType) | (q->s1_mask[g] ? kCtlS1 : 0) | (q->s2_mask && q->s2_mask[g] ? kCtlS2 : 0));
    }
    if (q->s1_onset) {
        on.resize(n);
        for (int64_t k = 0; k < n; ++k) on[k] = q->s1_onset[s->tm.cells[k]];
        if (!s->onset && s->mem.alloc((void **)&s->onset, n * 4)) return LQT_ERR_NOMEM;
        CK(cudaMemcpyAsync(s->onset, on.data(), n * 4, cudaMemcpyHostToDevice, s->stream));
    } else {
        s->onset = nullptr;
    }
    CK(cudaMemcpyAsync(s->ctl, c.data(), n, cudaMemcpyHostToDevice, s->stream));
    s->proto = *q;
    s->proto.s1_mask = nullptr;     // masks are folded into the control bytes
    s->proto.s2_mask = nullptr;
    s->proto.s1_onset = nullptr;
    s->has_s2 = q->s2_mask != nullptr;
    s->has_protocol = true;
    s->graph_valid = false;
    int rc = refresh_windows(s, s->step + 200000);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

// Enqueue nsteps steps on the simulation's stream (graph chunks where they
// fit, single steps elsewhere); the host does not wait for them.
static int sim_advance(lqt_sim *s, int64_t nsteps)
{
    if (s->has_protocol && s->step + nsteps + kGraphChunk > s->win_horizon) {
        int rc = refresh_windows(s, s->step + nsteps + 200000);
        if (rc) return rc;
    }
    int64_t left = nsteps;
    if (!s->tuned && left >= 64) {
        int64_t used = 0;
        int rc = autotune(s, 5, &used);
        if (rc) return rc;
        left -= used;
    }
    while (left > 0) {
        // graph replay for whole chunks starting on a chunk boundary
        if (left >= kGraphChunk && s->step % kGraphChunk == 0 &&
            (s->ecg_every <= 0 || kGraphChunk % s->ecg_every == 0)) {
            if (!s->graph_valid || s->graph_cur != s->cur) {
                int rc = build_graph(s);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(s->graph, s->stream));
            if (s->sur) {
                s->sur_launches += kGraphChunk / s->sur_nsub;   // chunks start on macro-step boundaries
                s->plist_valid = true;
            }
            s->step += kGraphChunk;
            for (int i = 0; i < kGraphChunk; ++i) s->time += s->p.dt;
            left -= kGraphChunk;
            continue;
        }
        int rc = step_once(s);
        if (rc) return rc;
        --left;
    }
    return LQT_OK;
}

int lqt_sim_step(lqt_sim *s, int64_t nsteps)
{
    if (!s || nsteps < 0) return fail(LQT_ERR_INVALID, "lqt_sim_step: NULL handle or nsteps < 0");
    const int rc = sim_advance(s, nsteps);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

int lqt_sim_step_async(lqt_sim *s, int64_t nsteps)
{
    if (!s || nsteps < 0) return fail(LQT_ERR_INVALID, "lqt_sim_step_async: NULL handle or nsteps < 0");
    return sim_advance(s, nsteps);
}

int lqt_sim_sync(lqt_sim *s)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_sync: NULL handle");
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

int lqt_sim_get_v(lqt_sim *s, void *v_host, int as_double)
{
    if (!s || !v_host) return fail(LQT_ERR_INVALID, "lqt_sim_get_v: NULL");
    const int64_t n = s->ntissue;
    const size_t esz = as_double ? 8 : 4;
    void *tmp = s->aos;
    if (!tmp) {
        if (s->mem.alloc((void **)&s->aos, n * 320)) return LQT_ERR_NOMEM;
        tmp = s->aos;
    }
    const int32_t *gi = s->dim > 1 ? s->gidx : nullptr;
    if (s->fp64()) {
        if (as_double) CK((launch_gather_v<double, double>((double *)s->vg[s->cur], gi, (double *)tmp, n, s->stream)));
        else CK((launch_gather_v<double, float>((double *)s->vg[s->cur], gi, (float *)tmp, n, s->stream)));
    } else {
        if (as_double) CK((launch_gather_v<float, double>((float *)s->vg[s->cur], gi, (double *)tmp, n, s->stream)));
        else CK((launch_gather_v<float, float>((float *)s->vg[s->cur], gi, (float *)tmp, n, s->stream)));
    }
    CK(cudaMemcpyAsync(v_host, tmp, n * esz, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

int lqt_sim_get_v_async(lqt_sim *s, void *v_host, int as_double)
{
    if (!s || !v_host) return fail(LQT_ERR_INVALID, "lqt_sim_get_v_async: NULL");
    const int64_t n = s->ntissue;
    const size_t esz = as_double ? 8 : 4;
    constexpr int nc = lqt_sim::kCopyStreams, ns = lqt_sim::kVSlots, nd = lqt_sim::kVDone;
    static_assert(nd > ns, "a slot's previous copy must still have its completion event");
    if (!s->copy_stream[0]) {
        for (int i = 0; i < ns; ++i)
            if (s->mem.alloc(&s->vslot[i], n * 8)) return LQT_ERR_NOMEM;
        for (int c = 0; c < nc; ++c) {
            CK(cudaStreamCreateWithFlags(&s->copy_stream[c], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&s->chunk_done[c], cudaEventDisableTiming));
        }
        CK(cudaEventCreateWithFlags(&s->gathered, cudaEventDisableTiming));
        for (int i = 0; i < nd; ++i) CK(cudaEventCreateWithFlags(&s->vdone[i], cudaEventDisableTiming));
    }
    const int64_t seq = s->v_issued;
    void *slot = s->vslot[seq % ns];
    cudaEvent_t done = s->vdone[seq % nd];
    // copy seq - nd used this completion event: the host waits for it before
    // the event is recorded again (so every copy older than the last nd is
    // known complete), and the gather waits for the slot's previous copy
    if (seq >= nd) CK(cudaEventSynchronize(done));
    if (seq >= ns) CK(cudaStreamWaitEvent(s->stream, s->vdone[(seq - ns) % nd], 0));
    const int32_t *gi = s->dim > 1 ? s->gidx : nullptr;
    if (s->fp64()) {
        if (as_double) CK((launch_gather_v<double, double>((double *)s->vg[s->cur], gi, (double *)slot, n, s->stream)));
        else CK((launch_gather_v<double, float>((double *)s->vg[s->cur], gi, (float *)slot, n, s->stream)));
    } else {
        if (as_double) CK((launch_gather_v<float, double>((float *)s->vg[s->cur], gi, (double *)slot, n, s->stream)));
        else CK((launch_gather_v<float, float>((float *)s->vg[s->cur], gi, (float *)slot, n, s->stream)));
    }
    CK(cudaEventRecord(s->gathered, s->stream));
    // nc chunks of whole 256-byte blocks (the last takes the rest), one per
    // stream, joined on stream 0 into the copy's completion event
    const size_t bytes = (size_t)n * esz;
    const size_t chunk = (bytes / nc + 255) / 256 * 256;
    for (int c = 0; c < nc; ++c) {
        const size_t off = std::min(bytes, c * chunk);
        const size_t len = std::min(bytes, off + chunk) - off;
        CK(cudaStreamWaitEvent(s->copy_stream[c], s->gathered, 0));
        if (len) CK(cudaMemcpyAsync((char *)v_host + off, (const char *)slot + off, len, cudaMemcpyDeviceToHost,
                                    s->copy_stream[c]));
        if (c > 0) {
            CK(cudaEventRecord(s->chunk_done[c], s->copy_stream[c]));
            CK(cudaStreamWaitEvent(s->copy_stream[0], s->chunk_done[c], 0));
        }
    }
    CK(cudaEventRecord(done, s->copy_stream[0]));
    s->v_issued = seq + 1;
    return LQT_OK;
}

int lqt_sim_wait_v(lqt_sim *s)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_wait_v: NULL");
    for (cudaStream_t c : s->copy_stream)
        if (c) CK(cudaStreamSynchronize(c));
    return LQT_OK;
}

int lqt_sim_wait_v_upto(lqt_sim *s, int64_t seq)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_wait_v_upto: NULL");
    if (seq < 0 || seq >= s->v_issued)
        return fail(LQT_ERR_INVALID, "lqt_sim_wait_v_upto: copy " + std::to_string(seq) + " not issued (" +
                                         std::to_string(s->v_issued) + " so far)");
    // copies complete in order (each one's chunks join on copy stream 0);
    // the ones older than the last kVDone were waited for at issue
    if (seq >= s->v_issued - lqt_sim::kVDone) CK(cudaEventSynchronize(s->vdone[seq % lqt_sim::kVDone]));
    return LQT_OK;
}

int lqt_sim_get_state(lqt_sim *s, double *state_host)
{
    if (!s || !state_host) return fail(LQT_ERR_INVALID, "lqt_sim_get_state: NULL");
    const int64_t n = s->ntissue;
    if (!s->aos && s->mem.alloc((void **)&s->aos, n * 320)) return LQT_ERR_NOMEM;
    // V: gather into the state-transfer V buffer, then unpack
    if (!s->vtmp && s->mem.alloc(&s->vtmp, n * 8)) return LQT_ERR_NOMEM;
    void *vtmp = s->vtmp;
    const int32_t *gi = s->dim > 1 ? s->gidx : nullptr;
    cudaError_t e;
    if (s->fp64()) {
        e = launch_gather_v<double, double>((double *)s->vg[s->cur], gi, (double *)vtmp, n, s->stream);
        if (e == cudaSuccess) e = launch_unpack<double>(SoA<double>{(double *)vtmp, s->conc, (double *)s->gate, s->ld}, s->aos, n, s->stream);
    } else {
        e = launch_gather_v<float, float>((float *)s->vg[s->cur], gi, (float *)vtmp, n, s->stream);
        if (e == cudaSuccess) e = launch_unpack<float>(SoA<float>{(float *)vtmp, s->conc, (float *)s->gate, s->ld}, s->aos, n, s->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(state_host, s->aos, n * 320, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("lqt_sim_get_state: ") + cudaGetErrorString(e));
    return LQT_OK;
}

int lqt_sim_set_state(lqt_sim *s, const double *state_host)
{
    if (!s || !state_host) return fail(LQT_ERR_INVALID, "lqt_sim_set_state: NULL");
    const int64_t n = s->ntissue;
    if (!s->aos && s->mem.alloc((void **)&s->aos, n * 320)) return LQT_ERR_NOMEM;
    if (!s->vtmp && s->mem.alloc(&s->vtmp, n * 8)) return LQT_ERR_NOMEM;
    void *vtmp = s->vtmp;
    const int32_t *gi = s->dim > 1 ? s->gidx : nullptr;
    const size_t rsz = s->fp64() ? 8 : 4;
    cudaError_t e = cudaMemcpyAsync(s->aos, state_host, n * 320, cudaMemcpyHostToDevice, s->stream);
    // empty voxels that are not mirrored are never read; zero both grids
    if (e == cudaSuccess) e = cudaMemsetAsync(s->vg[0], 0, s->ngrid * rsz, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->vg[1], 0, s->ngrid * rsz, s->stream);
    if (s->fp64()) {
        if (e == cudaSuccess) e = launch_pack<double>(s->aos, SoA<double>{(double *)vtmp, s->conc, (double *)s->gate, s->ld}, n, s->stream);
        if (e == cudaSuccess) e = launch_scatter_v<double>((double *)vtmp, gi, (double *)s->vg[s->cur], n, s->stream);
        if (e == cudaSuccess) e = launch_ghost<double>(s->dev<double>(), s->cur, s->stream);
    } else {
        if (e == cudaSuccess) e = launch_pack<float>(s->aos, SoA<float>{(float *)vtmp, s->conc, (float *)s->gate, s->ld}, n, s->stream);
        if (e == cudaSuccess) e = launch_scatter_v<float>((float *)vtmp, gi, (float *)s->vg[s->cur], n, s->stream);
        if (e == cudaSuccess) e = launch_ghost<float>(s->dev<float>(), s->cur, s->stream);
    }
    // launch_ghost also advanced the device clock: restore it
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("lqt_sim_set_state: ") + cudaGetErrorString(e));
    // a new state ends any macro step in progress: every voxel runs the plain
    // step until the next macro-step boundary
    if (s->srate) CK(cudaMemset(s->srate, 0xff, s->ntissue * 4));
    s->plist_valid = false;
    if (s->has_protocol) return refresh_windows(s, std::max<int64_t>(s->win_horizon, s->step + 1000));
    Clock c{};
    c.step = s->step;
    c.time = s->time;
    c.time_f = (float)s->time;
    c.s1_cycle_ok = 1;
    CK(cudaStreamSynchronize(s->stream));    // steps enqueued without waiting read the clock
    CK(cudaMemcpy(s->clk, &c, sizeof(c), cudaMemcpyHostToDevice));
    return LQT_OK;
}

int lqt_sim_set_electrodes(lqt_sim *s, int32_t n, const double *xyz, int32_t every)
{
    if (!s || n < 0 || n > kMaxElectrodes || (n > 0 && (!xyz || every <= 0)))
        return fail(LQT_ERR_INVALID, "lqt_sim_set_electrodes: 0..8 electrodes, every > 0");
    if (n > 0 && kGraphChunk % every != 0 && every % kGraphChunk != 0)
        return fail(LQT_ERR_INVALID, "lqt_sim_set_electrodes: `every` must divide 50 or be a multiple of 50");
    s->nel = n;
    s->ecg_every = every;
    s->graph_valid = false;
    if (n == 0) return LQT_OK;
    std::vector<float4> el(n);
    for (int i = 0; i < n; ++i) el[i] = make_float4((float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2], 0.f);
    if (!s->el) {
        int rc = s->mem.alloc((void **)&s->el, kMaxElectrodes * sizeof(float4)) |
                 s->mem.alloc((void **)&s->ecg_partial, ecg_blocks(s->ntissue) * kMaxElectrodes * 8) |
                 s->mem.alloc((void **)&s->ecg_count, 16);     // samples written, blocks done
        if (rc) return LQT_ERR_NOMEM;
    }
    s->ecg_cap = 1 << 16;
    if (!s->ecg_out) {
        int rc = s->mem.alloc((void **)&s->ecg_out, s->ecg_cap * kMaxElectrodes * 8) |
                 s->mem.alloc((void **)&s->ecg_t, s->ecg_cap * 8);
        if (rc) return LQT_ERR_NOMEM;
    }
    CK(cudaMemcpyAsync(s->el, el.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->ecg_count, 0, 16, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

int lqt_sim_get_ecg(lqt_sim *s, int64_t max_samples, double *phi, double *t, int64_t *nsamples)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_get_ecg: NULL");
    if (s->nel == 0) return fail(LQT_ERR_STATE, "lqt_sim_get_ecg: no electrodes set");
    int64_t cnt = 0;
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(&cnt, s->ecg_count, 8, cudaMemcpyDeviceToHost));
    if (nsamples) *nsamples = cnt;
    const int64_t m = std::min(cnt, max_samples);
    if (m > 0 && phi) {
        std::vector<double> buf(m * s->nel);
        CK(cudaMemcpy(buf.data(), s->ecg_out, m * s->nel * 8, cudaMemcpyDeviceToHost));
        std::memcpy(phi, buf.data(), m * s->nel * 8);
    }
    if (m > 0 && t) CK(cudaMemcpy(t, s->ecg_t, m * 8, cudaMemcpyDeviceToHost));
    return LQT_OK;
}

int lqt_sim_get_detect(lqt_sim *s, float *t_act, float *apd90, uint8_t *ead)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_get_detect: NULL");
    if (!s->det) return fail(LQT_ERR_STATE, "lqt_sim_get_detect: created with detect = 0");
    const int64_t n = s->ntissue;
    std::vector<float4> d(n);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(d.data(), s->det, n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < n; ++k) {
        uint32_t bits;
        std::memcpy(&bits, &d[k].w, 4);
        if (t_act) t_act[k] = d[k].z;
        if (ead) ead[k] = (bits >> 3) & 1u;
    }
    if (apd90) {
        CK(cudaMemcpy(apd90, s->apd90, n * 4, cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < n; ++k)
            if (!(apd90[k] == apd90[k])) apd90[k] = -1.f;
    }
    return LQT_OK;
}

int lqt_sim_tune(lqt_sim *s, int32_t variant, int32_t *chosen, float *ms_per_variant)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_tune: NULL handle");
    if (variant >= 0) {
        const int *cand = s->fp64() ? kGridVariantsF64 : kGridVariantsF32;
        const int ncand = s->fp64() ? 2 : 3;
        bool ok = false;
        for (int c = 0; c < ncand; ++c) ok |= cand[c] == variant;
        if (!ok) return fail(LQT_ERR_INVALID, "lqt_sim_tune: variant must be 2, 3 or 4 (mixed) or 1, 2 (FP64)");
        s->minb = variant;
        s->tuned = true;
        s->graph_valid = false;
    } else {
        int64_t used = 0;
        int rc = autotune(s, 5, &used);
        if (rc) return rc;
        CK(cudaStreamSynchronize(s->stream));
    }
    if (chosen) *chosen = s->minb;
    if (ms_per_variant) std::memcpy(ms_per_variant, s->tune_ms, sizeof(s->tune_ms));
    return LQT_OK;
}

int lqt_sim_substep_variant(lqt_sim *s, int32_t variant, int32_t *chosen, float *ms_per_variant)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_substep_variant: NULL handle");
    if (variant >= 0) {
        bool ok = false;
        for (int c = 0; c < kSubNVariants; ++c) ok |= kSubVariants[c] == variant;
        if (!ok) return fail(LQT_ERR_INVALID, "lqt_sim_substep_variant: variant must be 5, 6, 8, 105, 106 or 108");
        s->sub_minb = variant;
        s->sub_forced = true;
        s->graph_valid = false;
    }
    if (chosen) *chosen = s->sub_minb;
    if (ms_per_variant) std::memcpy(ms_per_variant, s->sub_tune_ms, sizeof(s->sub_tune_ms));
    return LQT_OK;
}

int lqt_sim_profile(lqt_sim *s, int64_t nsteps, double *ms_step, double *ms_ghost, double *ms_sur)
{
    if (!s || nsteps <= 0) return fail(LQT_ERR_INVALID, "lqt_sim_profile: NULL handle or nsteps <= 0");
    cudaEvent_t ev[5];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    double t_step = 0, t_ghost = 0, t_sur = 0;
    int64_t n_sur = 0;
    int rc = LQT_OK;
    for (int64_t i = 0; i < nsteps && rc == LQT_OK; ++i) {
        if (s->sur && s->step % s->sur_nsub == 0) {
            cudaError_t e = cudaEventRecord(ev[3], s->stream);
            if (e == cudaSuccess) rc = launch_sur_if_due(s);
            if (e == cudaSuccess && rc == LQT_OK) e = cudaEventRecord(ev[4], s->stream);
            if (e == cudaSuccess && rc == LQT_OK) e = cudaEventSynchronize(ev[4]);
            float ms = 0;
            if (e == cudaSuccess && rc == LQT_OK) e = cudaEventElapsedTime(&ms, ev[3], ev[4]);
            if (e != cudaSuccess) rc = fail(LQT_ERR_CUDA, std::string("lqt_sim_profile: ") + cudaGetErrorString(e));
            if (rc) break;
            t_sur += ms;
            ++n_sur;
        }
        cudaError_t e = cudaEventRecord(ev[0], s->stream);
        if (e == cudaSuccess) e = launch_substep(s);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], s->stream);
        if (e == cudaSuccess) e = launch_ghost_now(s);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2], s->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
        float a = 0, b = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&a, ev[0], ev[1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[1], ev[2]);
        if (e != cudaSuccess) rc = fail(LQT_ERR_CUDA, std::string("lqt_sim_profile: ") + cudaGetErrorString(e));
        t_step += a;
        t_ghost += b;
        s->cur ^= 1;
        s->step += 1;
        s->time += s->p.dt;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    if (ms_step) *ms_step = t_step / nsteps;
    if (ms_ghost) *ms_ghost = t_ghost / nsteps;
    if (ms_sur) *ms_sur = n_sur ? t_sur / n_sur : 0.0;
    return LQT_OK;
}

int lqt_sim_boundary(const lqt_sim *s, int64_t *dst, int64_t *src, int64_t *n)
{
    if (!s || !n) return fail(LQT_ERR_INVALID, "lqt_sim_boundary: NULL");
    *n = s->nbnd;
    if (dst) std::memcpy(dst, s->tm.bnd_dst.data(), s->nbnd * 8);
    if (src) std::memcpy(src, s->tm.bnd_src.data(), s->nbnd * 8);
    return LQT_OK;
}

int lqt_sim_check(lqt_sim *s, int64_t *n_bad)
{
    if (!s || !n_bad) return fail(LQT_ERR_INVALID, "lqt_sim_check: NULL");
    unsigned long long v = 0;
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(&v, s->nbad, sizeof(v), cudaMemcpyDeviceToHost));
    CK(cudaMemset(s->nbad, 0, sizeof(v)));
    *n_bad = (int64_t)v;
    if (s->sur_err) {
        int err = 0;
        CK(cudaMemcpy(&err, s->sur_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err & 2)
            return fail(LQT_ERR_CUDA, "lqt_sim_check: a surrogate substep's tile-copy wait ran out; voxels missed "
                                      "that substep and the run is not valid");
    }
    return v ? LQT_ERR_NUMERIC : LQT_OK;
}

int lqt_sim_sample_v(lqt_sim *s, int32_t stride, double *out_host, int64_t cap, int64_t *n)
{
    if (!s || !n || stride < 1) return fail(LQT_ERR_INVALID, "lqt_sim_sample_v: NULL or stride < 1");
    if (s->dim < 2) return fail(LQT_ERR_INVALID, "lqt_sim_sample_v: 2D and 3D grids only");
    const int64_t cnt = vtk_samples(s->nx, s->ny, s->nz, stride);
    *n = cnt;
    if (!out_host) return LQT_OK;
    if (cap < cnt) return fail(LQT_ERR_INVALID, "lqt_sim_sample_v: cap below the sample count");
    if (cnt > s->samp_cap) {
        if (s->samp) {
            cudaFree(s->samp);
            s->mem.ptrs.erase(std::remove(s->mem.ptrs.begin(), s->mem.ptrs.end(), (void *)s->samp), s->mem.ptrs.end());
            s->samp = nullptr;
        }
        if (s->mem.alloc((void **)&s->samp, cnt * 8)) return LQT_ERR_NOMEM;
        s->samp_cap = cnt;
    }
    int rc = sample_launch(s, stride, s->samp);
    if (rc) return rc;
    CK(cudaMemcpyAsync(out_host, s->samp, cnt * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LQT_OK;
}

int lqt_sim_set_surrogate(lqt_sim *s, lqt_mlp *m, const lqt_sur_config *cfg)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_set_surrogate: NULL handle");
    if (!m) {
        s->sur = nullptr;
        s->plist_valid = false;
        s->graph_valid = false;
        return LQT_OK;
    }
    if (s->fp64()) return fail(LQT_ERR_INVALID, "lqt_sim_set_surrogate: the surrogate runs in the mixed form only");
    if (s->p.model.dss_shift != 0.0 || s->p.model.fss_shift != 0.0 || s->p.model.suprep_dose > 0.0)
        return fail(LQT_ERR_INVALID, "lqt_sim_set_surrogate: the network's inputs carry the GKs, PCa and GKs-ISO "
                                     "factors only; models with ISO gate shifts or SUPREP are not covered");
    if (!cfg || !(cfg->dvdt_max > 0) || !(cfg->kappa > 0) || !(cfg->vstep_max > 0) ||
        !sur_nsub_ok(sur_nsub_or_default(cfg->nsub)) || (cfg->use_net != 0 && cfg->use_net != 1) ||
        !(cfg->foot_dvdt >= 0) || !std::isfinite(cfg->foot_v))
        return fail(LQT_ERR_INVALID, "lqt_sim_set_surrogate: dvdt_max, kappa, vstep_max > 0; use_net 0/1; "
                                     "nsub divides 50 (0 = 5); foot_dvdt >= 0; foot_v finite");
    MlpDev w;
    const float *nrm = nullptr;
    if (!mlp_device_view(m, &w, &nrm)) return fail(LQT_ERR_INVALID, "lqt_sim_set_surrogate: network not initialised");
    if (!s->srate) {
        int rc = s->mem.alloc((void **)&s->srate, pad_tiles(s->ntissue) * 4) |
                 s->mem.alloc((void **)&s->plist, s->ntissue * 4) |
                 s->mem.alloc((void **)&s->sdflag, pad_tiles(s->ntissue)) |
                 s->mem.alloc((void **)&s->plist_n, sizeof(unsigned long long)) |
                 s->mem.alloc((void **)&s->sur_stats, kSurNStats * sizeof(unsigned long long)) |
                 s->mem.alloc((void **)&s->sur_err, sizeof(int));
        if (rc) return LQT_ERR_NOMEM;
        CK(cudaMemsetAsync(s->sur_stats, 0, kSurNStats * sizeof(unsigned long long), s->stream));
        CK(cudaMemsetAsync(s->sdflag, 0, pad_tiles(s->ntissue), s->stream));
        CK(cudaMemsetAsync(s->sur_err, 0, sizeof(int), s->stream));
    }
    // the substep streams the tensor in FP16 (made once, padded to whole tiles)
    if (s->d6 && !s->t3h) {
        const int64_t np = pad_tiles(s->ntissue);
        if (s->mem.alloc((void **)&s->t3h, np * 12)) return LQT_ERR_NOMEM;
        CK(cudaMemsetAsync(s->t3h, 0, np * 12, s->stream));
        CK(launch_tensor_f16((const float *)s->d6, (const float *)s->b3, s->ntissue, (float)s->d_trans,
                             s->d_fibre >= s->d_trans ? 1.f : -1.f, s->t3h, s->stream));
    }
    // the V-halo boxes of the 3D substep (whole z-segments: nz a multiple of 4)
    if (s->d6 && s->dim == 3 && s->nz % 4 == 0 && !s->vbox_hdr) {
        std::vector<int32_t> hdr, li;
        build_vboxes(s->tm.cells, s->nx, s->ny, s->nz, hdr, li);
        if (s->mem.alloc((void **)&s->vbox_hdr, hdr.size() * 4) | s->mem.alloc((void **)&s->vli, li.size() * 4))
            return LQT_ERR_NOMEM;
        CK(cudaMemcpyAsync(s->vbox_hdr, hdr.data(), hdr.size() * 4, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->vli, li.data(), li.size() * 4, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    // NaN everywhere (the tile padding included): plain steps until the first
    // macro-step boundary
    CK(cudaMemsetAsync(s->srate, 0xff, pad_tiles(s->ntissue) * 4, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->sur = m;
    s->sur_cfg = *cfg;
    s->sur_nsub = sur_nsub_or_default(cfg->nsub);
    s->plist_valid = false;
    s->graph_valid = false;
    return LQT_OK;
}

int lqt_sim_set_wait_test(lqt_sim *s, int32_t skip_first_copy, uint32_t wait_limit)
{
    if (!s || (skip_first_copy != 0 && skip_first_copy != 1))
        return fail(LQT_ERR_INVALID, "lqt_sim_set_wait_test: NULL handle or skip_first_copy not 0/1");
    CK(cudaStreamSynchronize(s->stream));
    s->sub_skip_copy = skip_first_copy;
    s->sub_wait_limit = wait_limit;
    s->graph_valid = false;
    return LQT_OK;
}

int lqt_sim_surrogate_rejections(lqt_sim *s, int64_t *counts)
{
    if (!s || !counts) return fail(LQT_ERR_INVALID, "lqt_sim_surrogate_rejections: NULL argument");
    unsigned long long st[kSurNStats] = {};
    if (s->sur_stats) {
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaMemcpy(st, s->sur_stats, sizeof(st), cudaMemcpyDeviceToHost));
    }
    for (int r = 0; r < 4; ++r) counts[r] = (int64_t)st[2 + r];
    return LQT_OK;
}

int lqt_sim_surrogate_stats(lqt_sim *s, int64_t *macro_steps, int64_t *offered, int64_t *accepted,
                            int32_t *wait_timeouts, int32_t reset)
{
    if (!s) return fail(LQT_ERR_INVALID, "lqt_sim_surrogate_stats: NULL handle");
    unsigned long long st[2] = {0, 0};
    int err = 0;
    if (s->sur_stats) {
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaMemcpy(st, s->sur_stats, sizeof(st), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&err, s->sur_err, sizeof(int), cudaMemcpyDeviceToHost));
    }
    if (macro_steps) *macro_steps = s->sur_launches;
    if (offered) *offered = (int64_t)st[0];
    if (accepted) *accepted = (int64_t)st[1];
    if (wait_timeouts) *wait_timeouts = err;
    if (reset && s->sur_stats) {
        CK(cudaMemset(s->sur_stats, 0, kSurNStats * sizeof(unsigned long long)));
        CK(cudaMemset(s->sur_err, 0, sizeof(int)));
        s->sur_launches = 0;
    }
    return LQT_OK;
}

int lqt_sim_checkpoint(lqt_sim *s, const char *path)
{
    if (!s || !path) return fail(LQT_ERR_INVALID, "lqt_sim_checkpoint: NULL");
    std::vector<double> st((size_t)s->ntissue * 40);
    int rc = lqt_sim_get_state(s, st.data());
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(LQT_ERR_IO, std::string("lqt_sim_checkpoint: cannot open ") + path);
    const uint32_t hdr[4] = {kCkptMagic, kCkptVersion, (uint32_t)s->p.precision, (uint32_t)s->dim};
    const int64_t dims[4] = {s->nx, s->ny, s->nz, s->ntissue};
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(dims, sizeof(dims), 1, f) == 1 &&
              std::fwrite(&s->step, 8, 1, f) == 1 && std::fwrite(&s->time, 8, 1, f) == 1;
    // per-state arrays (state-major) so a field can be read without the rest
    std::vector<double> col(s->ntissue);
    for (int j = 0; j < 40 && ok; ++j) {
        for (int64_t k = 0; k < s->ntissue; ++k) col[k] = st[k * 40 + j];
        ok = std::fwrite(col.data(), 8, s->ntissue, f) == (size_t)s->ntissue;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? LQT_OK : fail(LQT_ERR_IO, "lqt_sim_checkpoint: write failed");
}

int lqt_sim_restore(lqt_sim *s, const char *path)
{
    if (!s || !path) return fail(LQT_ERR_INVALID, "lqt_sim_restore: NULL");
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(LQT_ERR_IO, std::string("lqt_sim_restore: cannot open ") + path);
    uint32_t hdr[4];
    int64_t dims[4], step = 0;
    double time = 0;
    bool ok = std::fread(hdr, sizeof(hdr), 1, f) == 1 && std::fread(dims, sizeof(dims), 1, f) == 1 &&
              std::fread(&step, 8, 1, f) == 1 && std::fread(&time, 8, 1, f) == 1;
    if (!ok || hdr[0] != kCkptMagic || hdr[1] != kCkptVersion) {
        std::fclose(f);
        return fail(LQT_ERR_IO, "lqt_sim_restore: not an lqt checkpoint (bad magic or version)");
    }
    if (dims[0] != s->nx || dims[1] != s->ny || dims[2] != s->nz || dims[3] != s->ntissue) {
        std::fclose(f);
        return fail(LQT_ERR_INVALID, "lqt_sim_restore: checkpoint geometry differs from this simulation");
    }
    std::vector<double> st((size_t)s->ntissue * 40), col(s->ntissue);
    for (int j = 0; j < 40 && ok; ++j) {
        ok = std::fread(col.data(), 8, s->ntissue, f) == (size_t)s->ntissue;
        for (int64_t k = 0; k < s->ntissue && ok; ++k) st[k * 40 + j] = col[k];
    }
    std::fclose(f);
    if (!ok) return fail(LQT_ERR_IO, "lqt_sim_restore: truncated checkpoint");
    s->step = step;
    s->time = time;
    s->graph_valid = false;
    return lqt_sim_set_state(s, st.data());
}

}  // extern "C"

// ===========================================================================
// Asynchronous VTK writer: the lattice is sampled on the device and copied
// into a pinned buffer on the simulation's stream; a host thread formats and
// writes the file once that copy has completed, while the simulation steps on.
struct lqt_vtk_writer {
    lqt_sim *s = nullptr;
    int32_t stride = 3;
    int64_t n = 0;
    std::vector<double *> dbuf, hbuf;
    std::vector<cudaEvent_t> ev;
    std::vector<bool> busy;
    std::deque<std::pair<int, std::string>> jobs;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    int err = LQT_OK;
    std::string errmsg;
    std::thread th;

    void run()
    {
        for (;;) {
            std::pair<int, std::string> job;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !jobs.empty(); });
                if (jobs.empty()) return;
                job = jobs.front();
                jobs.pop_front();
            }
            int rc = LQT_OK;
            std::string msg;
            if (cudaEventSynchronize(ev[job.first]) != cudaSuccess) {
                rc = LQT_ERR_CUDA;
                msg = "lqt_vtk_writer: device copy failed";
            } else {
                rc = write_vtk_file(job.second.c_str(), hbuf[job.first], s->nx, s->ny, s->nz, stride);
                if (rc) msg = g_err;
            }
            std::lock_guard<std::mutex> lk(mu);
            busy[job.first] = false;
            if (rc && err == LQT_OK) {
                err = rc;
                errmsg = msg;
            }
            cv.notify_all();
        }
    }
    ~lqt_vtk_writer()
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        if (th.joinable()) th.join();
        for (auto p : dbuf) if (p) cudaFree(p);
        for (auto p : hbuf) if (p) cudaFreeHost(p);
        for (auto e : ev) if (e) cudaEventDestroy(e);
    }
};

extern "C" {

int lqt_vtk_writer_create(lqt_sim *s, int32_t stride, int32_t nbuf, lqt_vtk_writer **out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_vtk_writer_create: out is NULL");
    *out = nullptr;
    if (!s || stride < 1 || nbuf < 1 || nbuf > 16)
        return fail(LQT_ERR_INVALID, "lqt_vtk_writer_create: NULL, stride < 1 or nbuf outside 1..16");
    if (s->dim < 2) return fail(LQT_ERR_INVALID, "lqt_vtk_writer_create: 2D and 3D grids only");
    auto *w = new lqt_vtk_writer();
    w->s = s;
    w->stride = stride;
    w->n = vtk_samples(s->nx, s->ny, s->nz, stride);
    w->dbuf.assign(nbuf, nullptr);
    w->hbuf.assign(nbuf, nullptr);
    w->ev.assign(nbuf, nullptr);
    w->busy.assign(nbuf, false);
    for (int i = 0; i < nbuf; ++i) {
        if (cudaMalloc((void **)&w->dbuf[i], w->n * 8) != cudaSuccess ||
            cudaHostAlloc((void **)&w->hbuf[i], w->n * 8, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&w->ev[i], cudaEventDisableTiming) != cudaSuccess) {
            delete w;
            return fail(LQT_ERR_NOMEM, "lqt_vtk_writer_create: buffer allocation failed");
        }
    }
    w->th = std::thread([w] { w->run(); });
    *out = w;
    return LQT_OK;
}

int lqt_vtk_writer_submit(lqt_vtk_writer *w, const char *path)
{
    if (!w || !path) return fail(LQT_ERR_INVALID, "lqt_vtk_writer_submit: NULL");
    int idx = -1;
    {
        std::unique_lock<std::mutex> lk(w->mu);
        w->cv.wait(lk, [&] {
            if (w->err) return true;
            for (size_t i = 0; i < w->busy.size(); ++i)
                if (!w->busy[i]) return true;
            return false;
        });
        if (w->err) return fail(w->err, w->errmsg);
        for (size_t i = 0; i < w->busy.size(); ++i)
            if (!w->busy[i]) {
                idx = (int)i;
                break;
            }
        w->busy[idx] = true;
    }
    lqt_sim *s = w->s;
    int rc = sample_launch(s, w->stride, w->dbuf[idx]);
    cudaError_t e = rc ? cudaSuccess : cudaMemcpyAsync(w->hbuf[idx], w->dbuf[idx], w->n * 8, cudaMemcpyDeviceToHost,
                                                       s->stream);
    if (!rc && e == cudaSuccess) e = cudaEventRecord(w->ev[idx], s->stream);
    std::lock_guard<std::mutex> lk(w->mu);
    if (rc || e != cudaSuccess) {
        w->busy[idx] = false;
        return rc ? rc : fail(LQT_ERR_CUDA, std::string("lqt_vtk_writer_submit: ") + cudaGetErrorString(e));
    }
    w->jobs.emplace_back(idx, std::string(path));
    w->cv.notify_all();
    return LQT_OK;
}

int lqt_vtk_writer_flush(lqt_vtk_writer *w)
{
    if (!w) return fail(LQT_ERR_INVALID, "lqt_vtk_writer_flush: NULL");
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] {
        if (!w->jobs.empty()) return false;
        for (bool b : w->busy)
            if (b) return false;
        return true;
    });
    if (w->err) {
        const int rc = w->err;
        w->err = LQT_OK;
        return fail(rc, w->errmsg);
    }
    return LQT_OK;
}

void lqt_vtk_writer_destroy(lqt_vtk_writer *w)
{
    if (!w) return;
    lqt_vtk_writer_flush(w);
    delete w;
}

}  // extern "C"
