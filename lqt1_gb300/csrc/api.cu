// api.cu -- host side of the C ABI (include/lqt.h): handles, validation,
// device memory, stimulus schedules and kernel launches.  No torch types.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lqt.h"
#include "api_common.h"
#include "lqt_internal.h"

namespace lqt {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

// SingleCell/TPORd.cc:142-198
void initial_state(double v0, double *s)
{
    static const double rest[LQT_NSTATE] = {
        -87.5, 7.0, 7.0, 145.0, 145.0, 1.0e-4, 1.0e-4, 1.2, 1.2,   // v, concentrations
        0.0, 1.0, 1.0, 1.0, 1.0,                                    // sm sh sj hsp jp
        0.0, 1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0,                // mL hL hLp a iF iS ap iFp iSp
        0.0, 1.0, 1.0, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0,                // d ff fs fcaf fcas jca nca ffp fcafp
        0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0};                    // xrf xrs xs1 xs2 xk1 Jrelnp Jrelp CaMKt
    std::memcpy(s, rest, sizeof(rest));
    s[0] = v0;
}

// Per-class PCa and GKs in the order of SingleCell/TPORd.cc:622-639 and
// 692-733 (GPU3D.cu:754-902 uses the same order).
ModelK make_modelk(const lqt_model &m)
{
    ModelK k{};
    for (int cls = 0; cls < 3; ++cls) {
        const bool epi = cls == 1, mid = cls == 2;
        double PCa = 0.0001;
        PCa *= m.pca_scale;
        if (epi) PCa *= 1.2;
        if (mid) PCa *= 2.5;
        k.pca[cls] = PCa;
        double GKs = 0.0034 * 1;
        if (epi) GKs *= 1.4;
        GKs = m.gks_scale * GKs;
        if (m.suprep_dose > 0.0) {
            const double dose = m.suprep_dose;
            const double GKs_sup = GKs;
            const double GKs_rep = epi ? 1.4 * 0.0034 : 0.0034;
            double frac_wt = 1.0;
            if (dose >= 25)
                frac_wt = 3.129 * std::pow(dose, -0.560);
            else
                frac_wt = std::pow(0.974, dose);
            const double frac_sh = 2.018 * (1.0 - std::exp(-2.0 * dose * 0.0059)) / (1.0 + std::exp(-2.0 * dose * 0.0059));
            GKs = frac_wt * GKs_sup + frac_sh * GKs_rep;
        }
        GKs *= m.gks_iso_scale;
        k.gks[cls] = GKs;
    }
    k.dss_shift = m.dss_shift;
    k.fss_shift = m.fss_shift;
    return k;
}

StepK make_stepk(double dt)
{
    StepK k;
    k.dt = dt;
    k.e_hl = std::exp(-dt / 200.0);      // thL = 200 (TPORd.cc:517)
    k.e_hlp = std::exp(-dt / (3.0 * 200.0));
    k.e_jca = std::exp(-dt / 75.0);      // tjca (TPORd.cc:605)
    return k;
}

int check_model(const lqt_model &m)
{
    if (!(m.pca_scale > 0) || !(m.gks_scale >= 0) || !(m.gks_iso_scale >= 0) || !std::isfinite(m.dss_shift) ||
        !std::isfinite(m.fss_shift) || !std::isfinite(m.suprep_dose) || m.reserved[0] != 0 || m.reserved[1] != 0)
        return fail(LQT_ERR_INVALID, "lqt_model: scales must be finite (pca > 0, gks >= 0), reserved must be 0");
    return LQT_OK;
}

// Shared time axis: time_k = sum of k additions of dt in FP64, exactly as
// `for (time = 0; ...; time += dt)` (OneD.cc:317, SingleCell.cc:95).
void time_axis(double dt, double t_stop, std::vector<double> &times)
{
    times.clear();
    double time = 0.0;
    while (time <= t_stop) {
        times.push_back(time);
        time += dt;
    }
}

// Window test of OneD.cc:337-338 / SingleCell.cc:98-99.
static inline bool in_window(double time, double bcl, double start, double dur)
{
    const double tb = time - std::floor(time / bcl) * bcl;
    return tb >= start && tb < start + dur;
}

// Step ranges [on, off) of the S1 windows within the first nsteps steps.
// The accumulated time differs from k*dt by far less than one step, so each
// edge is searched in a few steps around its nominal index.
void stim_windows(const std::vector<double> &times, int64_t nsteps, double dt, double bcl, double start, double dur,
                  int beats, std::vector<Win> &out)
{
    if (!(bcl > 0) || !(dur > 0) || nsteps <= 0) return;
    const double t_end = times[nsteps - 1];
    for (int64_t c = 0;; ++c) {
        if (beats > 0 && c >= beats) break;
        const double t_on = c * bcl + start;
        if (t_on > t_end + dt) break;
        int64_t k0 = (int64_t)std::floor(t_on / dt) - 4;
        if (k0 < 0) k0 = 0;
        int64_t on = -1;
        for (int64_t k = k0; k < std::min(nsteps, k0 + 12); ++k)
            if (in_window(times[k], bcl, start, dur) && (int64_t)std::floor(times[k] / bcl) == c) {
                on = k;
                break;
            }
        if (on < 0) continue;
        int64_t k1 = (int64_t)std::floor((t_on + dur) / dt) - 4;
        if (k1 <= on) k1 = on + 1;
        int64_t off = nsteps;
        for (int64_t k = k1; k < nsteps; ++k)
            if (!in_window(times[k], bcl, start, dur)) {
                off = k;
                break;
            }
        // every step between on and off is inside (the window is contiguous)
        out.push_back(Win{on, off});
    }
}

int64_t pad128(int64_t n) { return (n + 127) / 128 * 128; }

}  // namespace lqt

using namespace lqt;

// ===========================================================================
extern "C" {

const char *lqt_last_error(void) { return g_err.c_str(); }

int lqt_model_preset(int preset, lqt_model *out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_model_preset: out is NULL");
    lqt_model m{};
    m.pca_scale = m.gks_scale = m.gks_iso_scale = 1.0;
    switch (preset) {
    case LQT_PRESET_BASELINE:
    case LQT_PRESET_CON:
        break;
    case LQT_PRESET_CPU_DEFAULT:
        m.dss_shift = 12.0; m.fss_shift = 8.0; m.pca_scale = 1.6; m.gks_iso_scale = 3.2;
        break;
    case LQT_PRESET_LQT1:
    case LQT_PRESET_GPU2D:
        m.gks_scale = 0.05;
        break;
    case LQT_PRESET_GPU3D:
        m.dss_shift = 12.0; m.fss_shift = 8.0; m.pca_scale = 4.0; m.gks_scale = 0.05; m.gks_iso_scale = 3.2;
        m.suprep_dose = 100.0;
        break;
    default:
        return fail(LQT_ERR_INVALID, "lqt_model_preset: unknown preset");
    }
    *out = m;
    return LQT_OK;
}

int lqt_initial_state(double v0, double *state40_host)
{
    if (!state40_host) return fail(LQT_ERR_INVALID, "lqt_initial_state: NULL");
    initial_state(v0, state40_host);
    return LQT_OK;
}

}  // extern "C"

// ===========================================================================
// Cells (Cell interface for N cells)
struct lqt_cells {
    int precision = LQT_MIXED;
    int64_t n = 0, ld = 0;
    cudaStream_t stream = nullptr;
    DevMem mem;
    uint8_t *ctype = nullptr;
    double *ist = nullptr, *dvgap = nullptr, *dvdt = nullptr, *aos = nullptr, *cur = nullptr;
    void *v = nullptr, *gate = nullptr;
    double *conc = nullptr;
    ModelK *modelk = nullptr;
    StepK stepk{};
    template <typename R> SoA<R> soa() const { return SoA<R>{(R *)v, conc, (R *)gate, ld}; }
};

extern "C" {

int lqt_cells_create(int64_t n, const uint8_t *types_host, int precision, const lqt_model *model, double dt,
                     void *stream, lqt_cells **out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_cells_create: out is NULL");
    *out = nullptr;
    if (n <= 0 || !types_host || !model) return fail(LQT_ERR_INVALID, "lqt_cells_create: n <= 0 or NULL argument");
    if (precision != LQT_FP64 && precision != LQT_MIXED) return fail(LQT_ERR_INVALID, "lqt_cells_create: precision");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(LQT_ERR_INVALID, "lqt_cells_create: dt must be > 0");
    int rc = check_model(*model);
    if (rc) return rc;
    for (int64_t i = 0; i < n; ++i)
        if (types_host[i] > LQT_MCELL) return fail(LQT_ERR_INVALID, "lqt_cells_create: cell type out of range");
    auto *c = new lqt_cells();
    c->precision = precision;
    c->n = n;
    c->ld = pad128(n);
    c->stream = (cudaStream_t)stream;
    c->stepk = make_stepk(dt);
    const size_t rsz = precision == LQT_FP64 ? 8 : 4;
    rc = c->mem.alloc((void **)&c->ctype, n) | c->mem.alloc((void **)&c->ist, n * 8) |
         c->mem.alloc((void **)&c->dvgap, n * 8) | c->mem.alloc((void **)&c->dvdt, n * 8) |
         c->mem.alloc((void **)&c->cur, n * 6 * 8) |
         c->mem.alloc((void **)&c->aos, n * 40 * 8) | c->mem.alloc(&c->v, c->ld * rsz) |
         c->mem.alloc(&c->gate, c->ld * rsz * kNGate) | c->mem.alloc((void **)&c->conc, c->ld * 8 * kNConc) |
         c->mem.alloc((void **)&c->modelk, sizeof(ModelK));
    if (rc) {
        delete c;
        return fail(LQT_ERR_NOMEM, "lqt_cells_create: device allocation failed: " + g_err);
    }
    ModelK mk = make_modelk(*model);
    std::vector<double> init((size_t)n * 40);
    for (int64_t i = 0; i < n; ++i) initial_state(-87.5, &init[i * 40]);
    cudaError_t e = cudaMemcpyAsync(c->ctype, types_host, n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->modelk, &mk, sizeof(mk), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->ist, 0, n * 8, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dvgap, 0, n * 8, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dvdt, 0, n * 8, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->cur, 0, n * 6 * 8, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->aos, init.data(), n * 320, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = precision == LQT_FP64 ? launch_pack<double>(c->aos, c->soa<double>(), n, c->stream)
                                  : launch_pack<float>(c->aos, c->soa<float>(), n, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        delete c;
        return fail(LQT_ERR_CUDA, std::string("lqt_cells_create: ") + cudaGetErrorString(e));
    }
    *out = c;
    return LQT_OK;
}

void lqt_cells_destroy(lqt_cells *c) { delete c; }

int64_t lqt_cells_count(const lqt_cells *c) { return c ? c->n : -1; }

int lqt_cells_set_state(lqt_cells *c, const double *state_host)
{
    if (!c || !state_host) return fail(LQT_ERR_INVALID, "lqt_cells_set_state: NULL");
    CK(cudaMemcpyAsync(c->aos, state_host, c->n * 320, cudaMemcpyHostToDevice, c->stream));
    CK(c->precision == LQT_FP64 ? launch_pack<double>(c->aos, c->soa<double>(), c->n, c->stream)
                                : launch_pack<float>(c->aos, c->soa<float>(), c->n, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

int lqt_cells_get_state(lqt_cells *c, double *state_host)
{
    if (!c || !state_host) return fail(LQT_ERR_INVALID, "lqt_cells_get_state: NULL");
    CK(c->precision == LQT_FP64 ? launch_unpack<double>(c->soa<double>(), c->aos, c->n, c->stream)
                                : launch_unpack<float>(c->soa<float>(), c->aos, c->n, c->stream));
    CK(cudaMemcpyAsync(state_host, c->aos, c->n * 320, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

int lqt_cells_set_inputs(lqt_cells *c, const double *istim_host, const double *dvgap_host)
{
    if (!c) return fail(LQT_ERR_INVALID, "lqt_cells_set_inputs: NULL handle");
    if (istim_host) CK(cudaMemcpyAsync(c->ist, istim_host, c->n * 8, cudaMemcpyHostToDevice, c->stream));
    else CK(cudaMemsetAsync(c->ist, 0, c->n * 8, c->stream));
    if (dvgap_host) CK(cudaMemcpyAsync(c->dvgap, dvgap_host, c->n * 8, cudaMemcpyHostToDevice, c->stream));
    else CK(cudaMemsetAsync(c->dvgap, 0, c->n * 8, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

int lqt_cells_update(lqt_cells *c, int64_t nsteps)
{
    if (!c || nsteps < 0) return fail(LQT_ERR_INVALID, "lqt_cells_update: NULL handle or nsteps < 0");
    if (nsteps == 0) return LQT_OK;
    CK(c->precision == LQT_FP64
           ? launch_cells_update<double>(c->soa<double>(), c->ctype, c->ist, c->dvgap, c->dvdt, c->cur, c->modelk,
                                         nullptr, c->stepk, c->n, nsteps, c->stream)
           : launch_cells_update<float>(c->soa<float>(), c->ctype, c->ist, c->dvgap, c->dvdt, c->cur, c->modelk,
                                        nullptr, c->stepk, c->n, nsteps, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

int lqt_cells_get_v(lqt_cells *c, double *v_host)
{
    if (!c || !v_host) return fail(LQT_ERR_INVALID, "lqt_cells_get_v: NULL");
    std::vector<double> aos((size_t)c->n * 40);
    int rc = lqt_cells_get_state(c, aos.data());
    if (rc) return rc;
    for (int64_t i = 0; i < c->n; ++i) v_host[i] = aos[i * 40];
    return LQT_OK;
}

int lqt_cells_get_dvdt(lqt_cells *c, double *dvdt_host)
{
    if (!c || !dvdt_host) return fail(LQT_ERR_INVALID, "lqt_cells_get_dvdt: NULL");
    CK(cudaMemcpyAsync(dvdt_host, c->dvdt, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

int lqt_cells_get_currents(lqt_cells *c, double *currents_host)
{
    if (!c || !currents_host) return fail(LQT_ERR_INVALID, "lqt_cells_get_currents: NULL");
    CK(cudaMemcpyAsync(currents_host, c->cur, c->n * 6 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LQT_OK;
}

// ---- text state I/O (TPORd::outputAllStates / readinAllStates) -------------
int lqt_state_write_text(const double *state40, int64_t ncells, FILE *f)
{
    if (!state40 || !f || ncells < 0) return fail(LQT_ERR_INVALID, "lqt_state_write_text: NULL or ncells < 0");
    for (int64_t i = 0; i < 40 * ncells; ++i)
        if (fprintf(f, "%4.10f\n", state40[i]) < 0) return fail(LQT_ERR_IO, "lqt_state_write_text: write failed");
    return LQT_OK;
}

int lqt_state_read_text(double *state40, int64_t ncells, FILE *f)
{
    if (!state40 || !f || ncells < 0) return fail(LQT_ERR_INVALID, "lqt_state_read_text: NULL or ncells < 0");
    for (int64_t i = 0; i < 40 * ncells; ++i) {
        double value;
        if (fscanf(f, "%lf", &value) != 1)
            return fail(LQT_ERR_IO, "lqt_state_read_text: value " + std::to_string(i) + " missing or not a number");
        state40[i] = value;
    }
    return LQT_OK;
}

int lqt_cells_output_states(lqt_cells *c, int64_t first, int64_t count, FILE *f)
{
    if (!c || !f || first < 0 || count < 0 || first + count > c->n)
        return fail(LQT_ERR_INVALID, "lqt_cells_output_states: NULL, or cells outside [0, n)");
    std::vector<double> aos((size_t)c->n * 40);
    int rc = lqt_cells_get_state(c, aos.data());
    if (rc) return rc;
    return lqt_state_write_text(aos.data() + 40 * first, count, f);
}

int lqt_cells_readin_states(lqt_cells *c, int64_t first, int64_t count, FILE *f)
{
    if (!c || !f || first < 0 || count < 0 || first + count > c->n)
        return fail(LQT_ERR_INVALID, "lqt_cells_readin_states: NULL, or cells outside [0, n)");
    std::vector<double> aos((size_t)c->n * 40);
    int rc = lqt_cells_get_state(c, aos.data());
    if (rc) return rc;
    rc = lqt_state_read_text(aos.data() + 40 * first, count, f);
    if (rc) return rc;
    return lqt_cells_set_state(c, aos.data());
}

}  // extern "C"
