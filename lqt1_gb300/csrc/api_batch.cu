// api_batch.cu -- lqt_batch_*: uneven batches of single cells and strands in
// one persistent launch (k_batch.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "api_common.h"

using namespace lqt;

struct lqt_batch {
    lqt_batch_params p{};
    int64_t ncells = 0, ld = 0;
    int32_t ninst = 0;
    int threads = 128, ctas = 152;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.f;
    DevMem mem;
    std::vector<int64_t> perm;          // internal cell -> input cell
    std::vector<int> order;             // internal order of instances
    int max_strand = 1;
    int minb = 1;
    bool own_stream = false;
    std::vector<std::pair<std::pair<int, int>, float>> tuned;   // ((width, minb), probe ms)
    cudaGraphExec_t graph = nullptr;
    std::vector<lqt_instance> inst;
    std::vector<int64_t> inst_cell0;    // input order: first cell of each instance
    std::vector<int64_t> inst_internal0;// internal first cell of each instance
    std::vector<int32_t> rec_slot;      // per instance
    std::vector<int64_t> inst_nsteps;
    int64_t rec_cap = 0;
    int32_t rec_width = 0;
    // device
    void *v = nullptr, *gate = nullptr;
    double *conc = nullptr, *aos = nullptr;
    uint8_t *ctype = nullptr;
    double *coeff = nullptr, *dcoeff = nullptr;
    int32_t *seg_of = nullptr;
    Seg *segs = nullptr;
    Item *items = nullptr;
    int32_t nitems = 0;
    Win *win = nullptr;
    ModelK *models = nullptr;
    int *queue = nullptr;
    unsigned long long *nbad = nullptr;
    double *rec_v = nullptr, *rec_cur = nullptr;
    double *rec_t = nullptr, *ecg = nullptr;
    float *vmax = nullptr;
    float *det_t_act = nullptr, *det_apd90 = nullptr, *det_dvdt = nullptr;
    uint8_t *det_ead = nullptr;
    int32_t *det_beats = nullptr;

    ~lqt_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
    template <typename R> BatchDev<R> dev() const
    {
        BatchDev<R> b{};
        b.s = SoA<R>{(R *)v, conc, (R *)gate, ld};
        b.ctype = ctype;
        b.coeff = coeff;
        b.dcoeff = dcoeff;
        b.seg_of = seg_of;
        b.segs = segs;
        b.items = items;
        b.nitems = nitems;
        b.max_beats = p.max_beats;
        b.win = win;
        b.models = models;
        b.dt = p.dt;
        b.step_cap = 0;
        b.queue = queue;
        b.nbad = nbad;
        b.vmin_ok = -200.0;
        b.vmax_ok = 200.0;
        b.rec_every = p.rec_every;
        b.rec_cap = rec_cap;
        b.rec_width = rec_width;
        b.rec_v = rec_v;
        b.rec_cur = rec_cur;
        b.vmax = vmax;
        b.rec_t = rec_t;
        b.ecg = ecg;
        b.det_t_act = det_t_act;
        b.det_apd90 = det_apd90;
        b.det_dvdt = det_dvdt;
        b.det_ead = det_ead;
        b.det_beats = det_beats;
        return b;
    }
};

static int upload(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    if (bytes == 0) return LQT_OK;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return LQT_OK;
}

// Next-fit partition of the internal order into items of at most W cells;
// a recorded strand gets an item of its own (its pseudo-ECG is per item).
static std::vector<Item> make_items(const lqt_batch *b, int W)
{
    std::vector<Item> items;
    Item cur{};
    auto flush = [&]() {
        if (cur.ncells > 0) items.push_back(cur);
        cur = Item{};
    };
    for (int oi : b->order) {
        const lqt_instance &q = b->inst[oi];
        const bool own = q.record && q.ncells > 1;
        if (own || cur.ncells + q.ncells > W) flush();
        if (cur.ncells == 0) {
            cur.cell0 = b->inst_internal0[oi];
            cur.nsteps = 0;
            cur.ecg_seg = -1;
        }
        cur.ncells += q.ncells;
        cur.nsteps = std::max(cur.nsteps, b->inst_nsteps[oi]);
        if (own) {
            cur.ecg_seg = oi;
            flush();
        }
    }
    flush();
    return items;
}

static int set_items(lqt_batch *b, int W, int minb)
{
    std::vector<Item> items = make_items(b, W);
    CK(cudaMemcpyAsync(b->items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->nitems = (int32_t)items.size();
    b->threads = W;
    b->minb = minb;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = b->p.precision == LQT_FP64 ? batch_max_ctas_per_sm<double>(W, minb)
                                                  : batch_max_ctas_per_sm<float>(W, minb);
    b->ctas = b->p.ctas > 0 ? b->p.ctas : std::max(1, std::min(b->nitems, nsm * std::max(1, per_sm)));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return LQT_OK;
}

static int launch_run(lqt_batch *b, int64_t step_cap)
{
    cudaStream_t st = b->stream;
    CK(cudaMemsetAsync(b->queue, 0, sizeof(int), st));
    CK(cudaMemsetAsync(b->nbad, 0, sizeof(unsigned long long), st));
    if (b->p.max_beats > 0) {
        const int64_t nb = b->ncells * b->p.max_beats;
        CK(cudaMemsetAsync(b->det_t_act, 0xff, nb * 4, st));   // 0xffffffff = NaN -> reported as -1
        CK(cudaMemsetAsync(b->det_apd90, 0xff, nb * 4, st));
        CK(cudaMemsetAsync(b->det_dvdt, 0xff, nb * 4, st));
        CK(cudaMemsetAsync(b->det_ead, 0, b->ncells, st));
        CK(cudaMemsetAsync(b->det_beats, 0, b->ncells * 4, st));
    }
    if (b->p.precision == LQT_FP64) {
        BatchDev<double> d = b->dev<double>();
        d.step_cap = step_cap;
        CK(launch_batch<double>(d, make_stepk(b->p.dt), b->threads, b->minb, b->ctas, st));
    } else {
        BatchDev<float> d = b->dev<float>();
        d.step_cap = step_cap;
        CK(launch_batch<float>(d, make_stepk(b->p.dt), b->threads, b->minb, b->ctas, st));
    }
    return LQT_OK;
}

// Autotuner: every (CTA width, min CTAs/SM) variant that fits the longest
// strand runs a capped probe (the same cells x steps for all) from a snapshot
// of the state, which is restored afterwards; the fastest is kept.
static int tune_batch(lqt_batch *b)
{
    auto all = b->p.precision == LQT_FP64 ? batch_variants<double>() : batch_variants<float>();
    std::vector<std::pair<int, int>> cand;
    for (auto &v : all)
        if (v.first >= b->max_strand && (b->p.threads == 0 || v.first == b->p.threads)) cand.push_back(v);
    if (cand.empty()) return fail(LQT_ERR_INVALID, "no kernel variant fits the longest strand");
    if (cand.size() == 1) return set_items(b, cand[0].first, cand[0].second);
    const size_t rsz = b->p.precision == LQT_FP64 ? 8 : 4;
    const size_t bytes_v = b->ld * rsz, bytes_g = b->ld * rsz * kNGate, bytes_c = b->ld * 8 * kNConc;
    void *snap = nullptr;
    CK(cudaMalloc(&snap, bytes_v + bytes_g + bytes_c));
    char *sp = (char *)snap;
    cudaStream_t st = b->stream;
    int rc = LQT_OK;
    auto copy_all = [&](bool save) -> int {
        CK(cudaMemcpyAsync(save ? sp : b->v, save ? b->v : sp, bytes_v, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(save ? sp + bytes_v : b->gate, save ? b->gate : sp + bytes_v, bytes_g,
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(save ? sp + bytes_v + bytes_g : (char *)b->conc, save ? (char *)b->conc : sp + bytes_v + bytes_g,
                           bytes_c, cudaMemcpyDeviceToDevice, st));
        return LQT_OK;
    };
    int64_t max_ns = 0;
    for (auto ns : b->inst_nsteps) max_ns = std::max(max_ns, ns);
    const int64_t cap = std::min<int64_t>(max_ns, 400);
    rc = copy_all(true);
    float best = 1e30f;
    std::pair<int, int> pick = cand[0];
    b->tuned.clear();
    for (size_t c = 0; c < cand.size() && !rc; ++c) {
        rc = set_items(b, cand[c].first, cand[c].second);
        if (rc) break;
        rc = launch_run(b, 8);                 // warm the variant's module
        if (!rc) rc = copy_all(false);
        if (!rc) {
            cudaError_t e = cudaEventRecord(b->ev0, st);
            if (e == cudaSuccess) rc = launch_run(b, cap);
            if (!rc && e == cudaSuccess) e = cudaEventRecord(b->ev1, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
            if (e != cudaSuccess && !rc) rc = fail(LQT_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(e));
            b->tuned.push_back({cand[c], ms});
            if (!rc && ms < best) {
                best = ms;
                pick = cand[c];
            }
        }
        if (!rc) rc = copy_all(false);
    }
    if (!rc) rc = set_items(b, pick.first, pick.second);
    cudaStreamSynchronize(st);
    cudaFree(snap);
    return rc;
}

extern "C" {

int lqt_batch_create(const lqt_batch_params *params, int32_t ninst, const lqt_instance *inst,
                     const uint8_t *cell_types_host, const double *coeff_host, int32_t nmodels,
                     const lqt_model *models, lqt_batch **out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_batch_create: out is NULL");
    *out = nullptr;
    if (!params || ninst <= 0 || !inst || !cell_types_host || nmodels <= 0 || !models)
        return fail(LQT_ERR_INVALID, "lqt_batch_create: NULL argument or empty batch");
    const lqt_batch_params &p = *params;
    if (!(p.dt > 0) || !std::isfinite(p.dt)) return fail(LQT_ERR_INVALID, "lqt_batch_create: dt must be > 0");
    if (p.precision != LQT_FP64 && p.precision != LQT_MIXED) return fail(LQT_ERR_INVALID, "lqt_batch_create: precision");
    if (p.max_beats < 0 || p.max_beats > 4096) return fail(LQT_ERR_INVALID, "lqt_batch_create: max_beats");
    if (p.rec_every <= 0) return fail(LQT_ERR_INVALID, "lqt_batch_create: rec_every must be > 0");
    for (int i = 0; i < nmodels; ++i) {
        int rc = check_model(models[i]);
        if (rc) return rc;
    }
    int max_strand = 1;
    int64_t ncells = 0;
    double t_max = 0;
    for (int i = 0; i < ninst; ++i) {
        const lqt_instance &q = inst[i];
        if (q.ncells < 1 || q.ncells > 512 || q.model < 0 || q.model >= nmodels || q.n_stim < 0 ||
            !(q.t_stop >= 0) || !std::isfinite(q.t_stop) || !(q.bcl > 0) || q.s1_duration < 0 || q.s1_beats < 0 ||
            (q.ncells > 1 && !(q.dx > 0)) || q.t_stop > 1e7 || q.s2_ncells < 0 || q.s2_cell0 < 0 ||
            (q.s2_ncells > 0 && q.s2_cell0 + q.s2_ncells > q.ncells) || q.s2_duration < 0 || q.record < 0 ||
            q.record > 3 || q.reserved0 != 0 || q.reserved1 != 0)
            return fail(LQT_ERR_INVALID, "lqt_batch_create: instance " + std::to_string(i) +
                                             " invalid (ncells 1..512, model index, bcl > 0, t_stop, dx > 0, "
                                             "S2 cells inside the instance, record 0..3, reserved 0)");
        max_strand = std::max(max_strand, (int)q.ncells);
        ncells += q.ncells;
        t_max = std::max(t_max, q.t_stop);
    }
    for (int64_t i = 0; i < ncells; ++i)
        if (cell_types_host[i] > LQT_MCELL) return fail(LQT_ERR_INVALID, "lqt_batch_create: cell type out of range");

    auto *b = new lqt_batch();
    b->p = p;
    b->ninst = ninst;
    b->ncells = ncells;
    b->ld = pad128(ncells);
    b->stream = (cudaStream_t)p.stream;
    if (!b->stream) {
        // the run is captured as a CUDA graph: not on the legacy default stream
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete b;
            return fail(LQT_ERR_CUDA, "lqt_batch_create: cannot create a stream");
        }
        b->own_stream = true;
    }
    b->inst.assign(inst, inst + ninst);
    if (p.threads != 0 && p.threads != 128 && p.threads != 256 && p.threads != 512) {
        delete b;
        return fail(LQT_ERR_INVALID, "lqt_batch_create: threads must be 0 (autotune), 128, 256 or 512");
    }
    if (p.threads > 0 && max_strand > p.threads) {
        delete b;
        return fail(LQT_ERR_INVALID, "lqt_batch_create: a strand is longer than the CTA width");
    }

    // time axis and per-instance step counts / windows
    std::vector<double> times;
    time_axis(p.dt, t_max, times);
    b->inst_nsteps.resize(ninst);
    std::vector<std::vector<Win>> wins(ninst);
    for (int i = 0; i < ninst; ++i) {
        const lqt_instance &q = inst[i];
        int64_t ns = std::upper_bound(times.begin(), times.end(), q.t_stop) - times.begin();
        b->inst_nsteps[i] = ns;
        stim_windows(times, ns, p.dt, q.bcl, q.s1_start, q.s1_duration, q.s1_beats, wins[i]);
    }

    // Fixed internal order: recorded strands first (each gets its own item,
    // for its pseudo-ECG), then every instance by step count, longest first.
    // Items for a CTA width W are a next-fit partition of this order, so the
    // state layout does not depend on W and the autotuner can try widths.
    b->inst_cell0.resize(ninst);
    for (int i = 0, c0 = 0; i < ninst; ++i) {
        b->inst_cell0[i] = c0;
        c0 += inst[i].ncells;
    }
    std::vector<int> order(ninst);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const bool ra = inst[a].record && inst[a].ncells > 1, rc2 = inst[c].record && inst[c].ncells > 1;
        if (ra != rc2) return ra;
        if (b->inst_nsteps[a] != b->inst_nsteps[c]) return b->inst_nsteps[a] > b->inst_nsteps[c];
        return inst[a].ncells > inst[c].ncells;
    });
    b->order = order;
    std::vector<Seg> segs(ninst);
    std::vector<Win> allwin;
    b->inst_internal0.assign(ninst, 0);
    b->perm.resize(ncells);
    b->rec_slot.assign(ninst, -1);
    int32_t nrec_slots = 0;
    int64_t next_cell = 0;
    bool any_cur = false, any_vmax = false;
    for (int oi : order) {
        const lqt_instance &q = inst[oi];
        Seg sg{};
        sg.cell0 = next_cell;
        sg.nsteps = b->inst_nsteps[oi];
        sg.n = q.ncells;
        sg.n_stim = q.n_stim;
        sg.model = q.model;
        sg.win0 = (int32_t)allwin.size();
        sg.nwin = (int32_t)wins[oi].size();
        allwin.insert(allwin.end(), wins[oi].begin(), wins[oi].end());
        sg.dx = q.dx;
        sg.stim = q.s1_strength;
        sg.ecg_x0 = q.ecg_x0;
        sg.act_thr = (float)q.act_threshold;
        sg.rec_slot = -1;
        sg.rec_cur = (q.record & 2) ? 1 : 0;
        any_cur |= sg.rec_cur != 0;
        // S2 and the maximum-V watch on the same floating time axis as the
        // reference: t - base >= offset (OneD_VW.cc:273-275,340)
        sg.s2_on = sg.s2_off = sg.vmax_from = INT64_MAX;
        sg.s2_c0 = q.s2_cell0;
        sg.s2_n = q.s2_ncells;
        sg.s2_stim = q.s2_strength;
        if (q.s2_ncells > 0 || q.track_vmax) {
            for (int64_t k = 0; k < sg.nsteps; ++k) {
                const double rel = times[k] - q.s2_base;
                if (rel >= q.s2_offset) {
                    if (sg.vmax_from == INT64_MAX) sg.vmax_from = k;
                    if (rel < q.s2_offset + q.s2_duration) {
                        if (sg.s2_on == INT64_MAX) sg.s2_on = k;
                        sg.s2_off = k + 1;
                    }
                }
            }
            if (q.s2_ncells <= 0) sg.s2_on = sg.s2_off = INT64_MAX;
            if (!q.track_vmax) sg.vmax_from = INT64_MAX;
        }
        any_vmax |= q.track_vmax != 0;
        if (q.record) {
            sg.rec_slot = nrec_slots++;
            b->rec_slot[oi] = sg.rec_slot;
            b->rec_width = std::max(b->rec_width, (int32_t)q.ncells);
        }
        segs[oi] = sg;
        b->inst_internal0[oi] = next_cell;
        for (int j = 0; j < q.ncells; ++j) b->perm[next_cell + j] = b->inst_cell0[oi] + j;
        next_cell += q.ncells;
    }
    b->max_strand = max_strand;
    // segments are indexed by input instance; cell -> segment map (internal order)
    std::vector<int32_t> seg_of(ncells);
    for (int i = 0; i < ninst; ++i)
        for (int j = 0; j < inst[i].ncells; ++j) seg_of[b->inst_internal0[i] + j] = i;
    int64_t max_ns_all = 0;
    for (auto ns : b->inst_nsteps) max_ns_all = std::max(max_ns_all, ns);
    b->rec_cap = nrec_slots ? (max_ns_all + p.rec_every - 1) / p.rec_every : 0;
    // per-cell inputs in internal order; dD/dx per strand as OneD.cc:123-131
    std::vector<uint8_t> ct(ncells);
    std::vector<double> co(ncells), dco(ncells);
    for (int i = 0; i < ninst; ++i) {
        const int n = inst[i].ncells;
        const int64_t in0 = b->inst_cell0[i], it0 = b->inst_internal0[i];
        for (int j = 0; j < n; ++j) {
            ct[it0 + j] = cell_types_host[in0 + j];
            co[it0 + j] = coeff_host ? coeff_host[in0 + j] : 0.154;
        }
        for (int j = 0; j < n; ++j) {
            const double *cc = &co[it0];
            double dd;
            if (n == 1) dd = 0.0;
            else if (j == 0) dd = (cc[j + 1] - cc[j]) / inst[i].dx;
            else if (j == n - 1) dd = (cc[j] - cc[j - 1]) / inst[i].dx;
            else dd = (cc[j + 1] - cc[j - 1]) / (2.0 * inst[i].dx);
            dco[it0 + j] = dd;
        }
    }
    std::vector<ModelK> mk(nmodels);
    for (int i = 0; i < nmodels; ++i) mk[i] = make_modelk(models[i]);
    std::vector<double> init((size_t)ncells * 40);
    for (int64_t i = 0; i < ncells; ++i) initial_state(p.v0, &init[i * 40]);

    const size_t rsz = p.precision == LQT_FP64 ? 8 : 4;
    const int64_t ld = b->ld, nb = (int64_t)p.max_beats;
    int rc = 0;
    rc |= b->mem.alloc(&b->v, ld * rsz);
    rc |= b->mem.alloc(&b->gate, ld * rsz * kNGate);
    rc |= b->mem.alloc((void **)&b->conc, ld * 8 * kNConc);
    rc |= b->mem.alloc((void **)&b->aos, ncells * 320);
    rc |= b->mem.alloc((void **)&b->ctype, ncells);
    rc |= b->mem.alloc((void **)&b->coeff, ncells * 8);
    rc |= b->mem.alloc((void **)&b->dcoeff, ncells * 8);
    rc |= b->mem.alloc((void **)&b->seg_of, ncells * 4);
    rc |= b->mem.alloc((void **)&b->segs, ninst * sizeof(Seg));
    rc |= b->mem.alloc((void **)&b->items, ninst * sizeof(Item));
    rc |= b->mem.alloc((void **)&b->win, allwin.size() * sizeof(Win));
    rc |= b->mem.alloc((void **)&b->models, nmodels * sizeof(ModelK));
    rc |= b->mem.alloc((void **)&b->queue, 16);
    rc |= b->mem.alloc((void **)&b->nbad, 16);
    if (nrec_slots) {
        rc |= b->mem.alloc((void **)&b->rec_v, (size_t)nrec_slots * b->rec_cap * b->rec_width * 8);
        if (any_cur) rc |= b->mem.alloc((void **)&b->rec_cur, (size_t)nrec_slots * b->rec_cap * 2 * 8);
        rc |= b->mem.alloc((void **)&b->rec_t, (size_t)nrec_slots * b->rec_cap * 8);
        rc |= b->mem.alloc((void **)&b->ecg, (size_t)nrec_slots * b->rec_cap * 8);
    }
    if (any_vmax) rc |= b->mem.alloc((void **)&b->vmax, ncells * 4);
    if (nb > 0) {
        rc |= b->mem.alloc((void **)&b->det_t_act, ncells * nb * 4);
        rc |= b->mem.alloc((void **)&b->det_apd90, ncells * nb * 4);
        rc |= b->mem.alloc((void **)&b->det_dvdt, ncells * nb * 4);
        rc |= b->mem.alloc((void **)&b->det_ead, ncells);
        rc |= b->mem.alloc((void **)&b->det_beats, ncells * 4);
    }
    if (rc) {
        std::string m = g_err;
        delete b;
        return fail(LQT_ERR_NOMEM, "lqt_batch_create: " + m);
    }
    std::vector<double> init_int((size_t)ncells * 40);
    for (int64_t i = 0; i < ncells; ++i) std::memcpy(&init_int[i * 40], &init[b->perm[i] * 40], 320);
    cudaStream_t st = b->stream;
    rc = upload(b->ctype, ct.data(), ncells, st) | upload(b->coeff, co.data(), ncells * 8, st) |
         upload(b->dcoeff, dco.data(), ncells * 8, st) | upload(b->seg_of, seg_of.data(), ncells * 4, st) |
         upload(b->segs, segs.data(), ninst * sizeof(Seg), st) |
         upload(b->win, allwin.data(), allwin.size() * sizeof(Win), st) |
         upload(b->models, mk.data(), nmodels * sizeof(ModelK), st) |
         upload(b->aos, init_int.data(), ncells * 320, st);
    if (rc) {
        std::string m = g_err;
        delete b;
        return fail(LQT_ERR_CUDA, m);
    }
    cudaError_t e = p.precision == LQT_FP64
                        ? launch_pack<double>(b->aos, SoA<double>{(double *)b->v, b->conc, (double *)b->gate, ld}, ncells, st)
                        : launch_pack<float>(b->aos, SoA<float>{(float *)b->v, b->conc, (float *)b->gate, ld}, ncells, st);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        delete b;
        return fail(LQT_ERR_CUDA, std::string("lqt_batch_create: ") + cudaGetErrorString(e));
    }
    rc = tune_batch(b);
    if (rc) {
        std::string m = g_err;
        delete b;
        return fail(rc, "lqt_batch_create: " + m);
    }
    *out = b;
    return LQT_OK;
}

void lqt_batch_destroy(lqt_batch *b) { delete b; }

int64_t lqt_batch_num_cells(const lqt_batch *b) { return b ? b->ncells : -1; }

int lqt_batch_run(lqt_batch *b)
{
    if (!b) return fail(LQT_ERR_INVALID, "lqt_batch_run: NULL handle");
    cudaStream_t st = b->stream;
    if (!b->graph) {
        // the whole run (resets + one persistent launch) as one CUDA graph
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = launch_run(b, 0);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("lqt_batch_run capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("lqt_batch_run instantiate: ") + cudaGetErrorString(e));
    }
    CK(cudaEventRecord(b->ev0, st));
    CK(cudaGraphLaunch(b->graph, st));
    CK(cudaEventRecord(b->ev1, st));
    CK(cudaEventSynchronize(b->ev1));
    CK(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
    return LQT_OK;
}

int lqt_batch_config(const lqt_batch *b, int32_t *threads, int32_t *minb, int32_t *ctas, int32_t *nitems)
{
    if (!b) return fail(LQT_ERR_INVALID, "lqt_batch_config: NULL handle");
    if (threads) *threads = b->threads;
    if (minb) *minb = b->minb;
    if (ctas) *ctas = b->ctas;
    if (nitems) *nitems = b->nitems;
    return LQT_OK;
}

double lqt_batch_last_run_ms(const lqt_batch *b) { return b ? b->last_ms : -1.0; }

int64_t lqt_batch_num_bad(lqt_batch *b)
{
    if (!b) return -1;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, b->nbad, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return (int64_t)n;
}

int lqt_batch_get_detect(lqt_batch *b, float *t_act, float *apd90, float *dvdt_max, uint8_t *ead, int32_t *nbeats)
{
    if (!b) return fail(LQT_ERR_INVALID, "lqt_batch_get_detect: NULL handle");
    if (b->p.max_beats == 0) return fail(LQT_ERR_STATE, "lqt_batch_get_detect: created with max_beats = 0");
    const int64_t n = b->ncells, nb = b->p.max_beats;
    std::vector<float> buf((size_t)(n * nb));
    auto fetch_f = [&](float *dst, const float *src) -> int {
        if (!dst) return LQT_OK;
        CK(cudaMemcpy(buf.data(), src, n * nb * 4, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = 0; k < nb; ++k) {
                float x = buf[i * nb + k];
                dst[b->perm[i] * nb + k] = (x == x) ? x : -1.f;
            }
        return LQT_OK;
    };
    int rc = fetch_f(t_act, b->det_t_act);
    if (!rc) rc = fetch_f(apd90, b->det_apd90);
    if (!rc) rc = fetch_f(dvdt_max, b->det_dvdt);
    if (rc) return rc;
    if (ead) {
        std::vector<uint8_t> e(n);
        CK(cudaMemcpy(e.data(), b->det_ead, n, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i) ead[b->perm[i]] = e[i];
    }
    if (nbeats) {
        std::vector<int32_t> e(n);
        CK(cudaMemcpy(e.data(), b->det_beats, n * 4, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i) nbeats[b->perm[i]] = e[i];
    }
    return LQT_OK;
}

int lqt_batch_get_record(lqt_batch *b, int32_t i, double *v, double *t, double *ecg, int64_t cap, int64_t *nrec)
{
    if (!b || i < 0 || i >= b->ninst) return fail(LQT_ERR_INVALID, "lqt_batch_get_record: bad handle or instance");
    const int slot = b->rec_slot[i];
    if (slot < 0) return fail(LQT_ERR_STATE, "lqt_batch_get_record: instance was not recorded");
    const int64_t ns = b->inst_nsteps[i];
    const int64_t nr = std::min<int64_t>((ns + b->p.rec_every - 1) / b->p.rec_every, b->rec_cap);
    if (nrec) *nrec = nr;
    const int64_t m = std::min(nr, cap);
    const int n = b->inst[i].ncells;
    if (v && m > 0) {
        std::vector<double> buf((size_t)(m * b->rec_width));
        CK(cudaMemcpy(buf.data(), b->rec_v + (int64_t)slot * b->rec_cap * b->rec_width, m * b->rec_width * 8,
                      cudaMemcpyDeviceToHost));
        for (int64_t r = 0; r < m; ++r) std::memcpy(v + r * n, &buf[r * b->rec_width], n * 8);
    }
    if (t && m > 0) CK(cudaMemcpy(t, b->rec_t + (int64_t)slot * b->rec_cap, m * 8, cudaMemcpyDeviceToHost));
    if (ecg && m > 0) CK(cudaMemcpy(ecg, b->ecg + (int64_t)slot * b->rec_cap, m * 8, cudaMemcpyDeviceToHost));
    return LQT_OK;
}

int lqt_batch_get_record_currents(lqt_batch *b, int32_t i, double *ical, double *iks, int64_t cap, int64_t *nrec)
{
    if (!b || i < 0 || i >= b->ninst) return fail(LQT_ERR_INVALID, "lqt_batch_get_record_currents: bad handle or instance");
    const int slot = b->rec_slot[i];
    if (slot < 0 || !(b->inst[i].record & 2) || !b->rec_cur)
        return fail(LQT_ERR_STATE, "lqt_batch_get_record_currents: instance was not recorded with currents");
    const int64_t ns = b->inst_nsteps[i];
    const int64_t nr = std::min<int64_t>((ns + b->p.rec_every - 1) / b->p.rec_every, b->rec_cap);
    if (nrec) *nrec = nr;
    const int64_t m = std::min(nr, cap);
    if (m > 0 && (ical || iks)) {
        std::vector<double> buf((size_t)m * 2);
        CK(cudaMemcpy(buf.data(), b->rec_cur + (int64_t)slot * b->rec_cap * 2, m * 16, cudaMemcpyDeviceToHost));
        for (int64_t r = 0; r < m; ++r) {
            if (ical) ical[r] = buf[2 * r];
            if (iks) iks[r] = buf[2 * r + 1];
        }
    }
    return LQT_OK;
}

int lqt_batch_get_vmax(lqt_batch *b, float *vmax_host)
{
    if (!b || !vmax_host) return fail(LQT_ERR_INVALID, "lqt_batch_get_vmax: NULL");
    if (!b->vmax) return fail(LQT_ERR_STATE, "lqt_batch_get_vmax: no instance has track_vmax set");
    std::vector<float> buf((size_t)b->ncells);
    CK(cudaMemcpy(buf.data(), b->vmax, b->ncells * 4, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < b->ncells; ++i) vmax_host[b->perm[i]] = buf[i];
    return LQT_OK;
}

int lqt_batch_get_state(lqt_batch *b, double *state_host)
{
    if (!b || !state_host) return fail(LQT_ERR_INVALID, "lqt_batch_get_state: NULL");
    cudaStream_t st = b->stream;
    const int64_t ld = b->ld;
    CK(b->p.precision == LQT_FP64
           ? launch_unpack<double>(SoA<double>{(double *)b->v, b->conc, (double *)b->gate, ld}, b->aos, b->ncells, st)
           : launch_unpack<float>(SoA<float>{(float *)b->v, b->conc, (float *)b->gate, ld}, b->aos, b->ncells, st));
    std::vector<double> buf((size_t)b->ncells * 40);
    CK(cudaMemcpyAsync(buf.data(), b->aos, b->ncells * 320, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int64_t i = 0; i < b->ncells; ++i) std::memcpy(state_host + b->perm[i] * 40, &buf[i * 40], 320);
    return LQT_OK;
}

int lqt_batch_set_state(lqt_batch *b, const double *state_host)
{
    if (!b || !state_host) return fail(LQT_ERR_INVALID, "lqt_batch_set_state: NULL");
    cudaStream_t st = b->stream;
    const int64_t ld = b->ld;
    std::vector<double> buf((size_t)b->ncells * 40);
    for (int64_t i = 0; i < b->ncells; ++i) std::memcpy(&buf[i * 40], state_host + b->perm[i] * 40, 320);
    CK(cudaMemcpyAsync(b->aos, buf.data(), b->ncells * 320, cudaMemcpyHostToDevice, st));
    CK(b->p.precision == LQT_FP64
           ? launch_pack<double>(b->aos, SoA<double>{(double *)b->v, b->conc, (double *)b->gate, ld}, b->ncells, st)
           : launch_pack<float>(b->aos, SoA<float>{(float *)b->v, b->conc, (float *)b->gate, ld}, b->ncells, st));
    CK(cudaStreamSynchronize(st));
    return LQT_OK;
}

}  // extern "C"
