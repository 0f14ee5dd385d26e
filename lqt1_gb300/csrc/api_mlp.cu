// api_mlp.cu -- lqt_mlp_*: the learned surrogate's network (mlp.h): weights,
// normalisation, tcgen05 inference and one training step (forward, MSE
// gradient, backward, Adam) on device buffers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "api_common.h"
#include "mlp.h"

using namespace lqt;

namespace lqt {
cudaError_t launch_mse_grad(const float *Y, const float *T, int64_t B, int nvalid, __nv_bfloat16 *dY, double *loss,
                            cudaStream_t st);
cudaError_t launch_colsum(const __nv_bfloat16 *X, int64_t B, int N, float *g, cudaStream_t st);
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, __nv_bfloat16 *pb, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, cudaStream_t st);
}  // namespace lqt

namespace {
// parameter block layout (FP32 master and BF16 copy share offsets)
constexpr int64_t kOW1 = 0, kOB1 = kOW1 + kMlpHid * kMlpIn;
constexpr int64_t kOW2 = kOB1 + kMlpHid, kOB2 = kOW2 + kMlpHid * kMlpHid;
constexpr int64_t kOW3 = kOB2 + kMlpHid, kOB3 = kOW3 + kMlpOut * kMlpHid;
constexpr int64_t kNParam = kOB3 + kMlpOut;
}  // namespace

struct lqt_mlp {
    cudaStream_t stream = nullptr;
    DevMem mem;
    float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;
    __nv_bfloat16 *Pb = nullptr;
    __nv_bfloat16 *W2t = nullptr, *W3t = nullptr;   // transposed BF16 weights for the data gradients
    float *norm = nullptr;          // in_mean[48], in_scale[48], out_scale[48], out_bound[48]
    int *err = nullptr;
    double *loss = nullptr;
    int64_t adam_t = 0;
    int nvalid = kMlpNState;
    int layout = 0;                 // descriptor stride-field assignment (0 = LBO along K)
    // training workspace
    int64_t ws_batch = 0;
    float *Z1 = nullptr, *Z2 = nullptr, *Y = nullptr;
    __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *dY = nullptr, *dZ1 = nullptr, *dZ2 = nullptr;
    float *Gpart = nullptr;         // split-K slices of the weight gradients (ordered reduction)
    DevMem ws;
    MlpDev dev() const
    {
        return MlpDev{Pb + kOW1, Pb + kOW2, Pb + kOW3, P + kOB1, P + kOB2, P + kOB3, P + kOW2, P + kOW3};
    }
};

namespace lqt {
bool mlp_device_view(const lqt_mlp *m, MlpDev *w, const float **norm)
{
    if (!m || !m->P || !m->Pb || !m->norm) return false;
    *w = m->dev();
    *norm = m->norm;
    return true;
}
}  // namespace lqt

static int upload_params(lqt_mlp *m, const std::vector<float> &p)
{
    std::vector<__nv_bfloat16> pb(p.size());
    for (size_t i = 0; i < p.size(); ++i) pb[i] = __float2bfloat16(p[i]);
    CK(cudaMemcpyAsync(m->P, p.data(), p.size() * 4, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemcpyAsync(m->Pb, pb.data(), pb.size() * 2, cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemsetAsync(m->M, 0, kNParam * 4, m->stream));
    CK(cudaMemsetAsync(m->V, 0, kNParam * 4, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    m->adam_t = 0;
    return LQT_OK;
}

// K slices of the weight-gradient GEMMs (K = batch): 64 rows (one staging
// chunk) each, at most 128 slices, so that the three GEMMs fill the SMs.
static int splitk_for(int64_t B) { return (int)std::min<int64_t>(128, std::max<int64_t>(1, B / 64)); }

static int ensure_ws(lqt_mlp *m, int64_t B)
{
    if (B <= m->ws_batch) return LQT_OK;
    m->ws.reset();
    int rc = m->ws.alloc((void **)&m->Z1, B * kMlpHid * 4) | m->ws.alloc((void **)&m->Z2, B * kMlpHid * 4) |
             m->ws.alloc((void **)&m->Y, B * kMlpOut * 4) | m->ws.alloc((void **)&m->H1, B * kMlpHid * 2) |
             m->ws.alloc((void **)&m->H2, B * kMlpHid * 2) | m->ws.alloc((void **)&m->dY, B * kMlpOut * 2) |
             m->ws.alloc((void **)&m->dZ1, B * kMlpHid * 2) | m->ws.alloc((void **)&m->dZ2, B * kMlpHid * 2) |
             m->ws.alloc((void **)&m->Gpart,
                         (int64_t)std::max(1, gemm_splitk_slices((int)B, splitk_for(B))) * kMlpHid * kMlpHid * 4);
    if (rc) return LQT_ERR_NOMEM;
    m->ws_batch = B;
    return LQT_OK;
}

static GemmArgs gemm(const __nv_bfloat16 *A, int64_t lda, int ta, const __nv_bfloat16 *B, int64_t ldb, int tb, int M,
                     int N, int K)
{
    GemmArgs g{};
    g.A = A;
    g.B = B;
    g.err = nullptr;
    g.lda = lda;
    g.ldb = ldb;
    g.ta = ta;
    g.tb = tb;
    g.M = M;
    g.N = N;
    g.K = K;
    return g;
}

// Forward + MSE gradient + backward into m->G (no update).
static int forward_backward(lqt_mlp *m, const __nv_bfloat16 *X, const float *T, int64_t B)
{
    // every GEMM reports a tensor-core wait that ran out in m->err (checked
    // where the host waits: lqt_mlp_gradients, lqt_mlp_train_step with a
    // loss, lqt_mlp_get_params)
    if (B <= 0 || B % 16 != 0 || B > (int64_t)INT32_MAX) return fail(LQT_ERR_INVALID, "batch must be a positive multiple of 16");
    int rc = ensure_ws(m, B);
    if (rc) return rc;
    cudaStream_t st = m->stream;
    const int b = (int)B;
    const __nv_bfloat16 *W1 = m->Pb + kOW1, *W2 = m->Pb + kOW2, *W3 = m->Pb + kOW3;
    GemmArgs g = gemm(X, kMlpIn, 0, W1, kMlpIn, 1, b, kMlpHid, kMlpIn);
    g.epi = kEpiStore; g.bias = m->P + kOB1; g.C = m->Z1; g.Cb = m->H1; g.act = 1;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    g = gemm(m->H1, kMlpHid, 0, W2, kMlpHid, 1, b, kMlpHid, kMlpHid);
    g.epi = kEpiStore; g.bias = m->P + kOB2; g.C = m->Z2; g.Cb = m->H2; g.act = 1;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    g = gemm(m->H2, kMlpHid, 0, W3, kMlpHid, 1, b, kMlpOut, kMlpHid);
    g.epi = kEpiStore; g.bias = m->P + kOB3; g.C = m->Y;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    CK(cudaMemsetAsync(m->loss, 0, 8, st));
    CK(launch_mse_grad(m->Y, T, B, m->nvalid, m->dY, m->loss, st));
    // data gradients: W^T as N x K operands with K contiguous
    CK(launch_transpose_w(W2, W3, m->W2t, m->W3t, st));
    g = gemm(m->dY, kMlpOut, 0, m->W3t, kMlpOut, 1, b, kMlpHid, kMlpOut);
    g.epi = kEpiDact; g.Z = m->Z2; g.Cb = m->dZ2;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    g = gemm(m->dZ2, kMlpHid, 0, m->W2t, kMlpHid, 1, b, kMlpHid, kMlpHid);
    g.epi = kEpiDact; g.Z = m->Z1; g.Cb = m->dZ1;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    CK(cudaMemsetAsync(m->G, 0, kNParam * 4, st));
    const int ks = splitk_for(B);
    g = gemm(m->dY, kMlpOut, 1, m->H2, kMlpHid, 0, kMlpOut, kMlpHid, b);
    g.epi = kEpiAtomic; g.C = m->G + kOW3; g.ksplit = ks; g.partial = m->Gpart;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    g = gemm(m->dZ2, kMlpHid, 1, m->H1, kMlpHid, 0, kMlpHid, kMlpHid, b);
    g.epi = kEpiAtomic; g.C = m->G + kOW2; g.ksplit = ks; g.partial = m->Gpart;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    g = gemm(m->dZ1, kMlpHid, 1, X, kMlpIn, 0, kMlpHid, kMlpIn, b);
    g.epi = kEpiAtomic; g.C = m->G + kOW1; g.ksplit = ks; g.partial = m->Gpart;
    g.err = m->err;
    CK(launch_gemm_bf16(g, st));
    CK(launch_colsum(m->dY, B, kMlpOut, m->G + kOB3, st));
    CK(launch_colsum(m->dZ2, B, kMlpHid, m->G + kOB2, st));
    CK(launch_colsum(m->dZ1, B, kMlpHid, m->G + kOB1, st));
    return LQT_OK;
}

extern "C" {

int lqt_mlp_create(uint64_t seed, void *stream, lqt_mlp **out)
{
    if (!out) return fail(LQT_ERR_INVALID, "lqt_mlp_create: out is NULL");
    auto *m = new lqt_mlp();
    m->stream = (cudaStream_t)stream;
    int rc = m->mem.alloc((void **)&m->P, kNParam * 4) | m->mem.alloc((void **)&m->G, kNParam * 4) |
             m->mem.alloc((void **)&m->M, kNParam * 4) | m->mem.alloc((void **)&m->V, kNParam * 4) |
             m->mem.alloc((void **)&m->Pb, kNParam * 2) | m->mem.alloc((void **)&m->norm, 4 * kMlpIn * 4) |
             m->mem.alloc((void **)&m->W2t, kMlpHid * kMlpHid * 2) |
             m->mem.alloc((void **)&m->W3t, kMlpHid * kMlpOut * 2) |
             m->mem.alloc((void **)&m->err, 16) | m->mem.alloc((void **)&m->loss, 16);
    if (rc) {
        delete m;
        return fail(LQT_ERR_NOMEM, "lqt_mlp_create: device allocation failed");
    }
    // He-style initialisation (fan-in), zero biases
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> N01(0.f, 1.f);
    std::vector<float> p(kNParam, 0.f);
    for (int64_t i = 0; i < kMlpHid * kMlpIn; ++i) p[kOW1 + i] = N01(rng) * std::sqrt(2.f / kMlpIn);
    for (int64_t i = 0; i < kMlpHid * kMlpHid; ++i) p[kOW2 + i] = N01(rng) * std::sqrt(2.f / kMlpHid);
    for (int64_t i = 0; i < kMlpOut * kMlpHid; ++i) p[kOW3 + i] = N01(rng) * std::sqrt(1.f / kMlpHid);
    rc = upload_params(m, p);
    std::vector<float> nrm(4 * kMlpIn, 0.f);
    for (int i = 0; i < kMlpIn; ++i) {
        nrm[kMlpIn + i] = nrm[2 * kMlpIn + i] = 1.f;
        nrm[3 * kMlpIn + i] = INFINITY;       // no residual bound until one is set
    }
    if (!rc && cudaMemcpy(m->norm, nrm.data(), nrm.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = LQT_ERR_CUDA;
    if (!rc && cudaMemset(m->err, 0, 16) != cudaSuccess) rc = LQT_ERR_CUDA;
    if (rc) {
        delete m;
        return fail(rc, "lqt_mlp_create: upload failed");
    }
    *out = m;
    return LQT_OK;
}

void lqt_mlp_destroy(lqt_mlp *m) { delete m; }

int64_t lqt_mlp_num_params(void) { return kNParam; }

int lqt_mlp_set_params(lqt_mlp *m, const float *params_host)
{
    if (!m || !params_host) return fail(LQT_ERR_INVALID, "lqt_mlp_set_params: NULL");
    std::vector<float> p(params_host, params_host + kNParam);
    for (float x : p)
        if (!std::isfinite(x)) return fail(LQT_ERR_INVALID, "lqt_mlp_set_params: non-finite parameter");
    return upload_params(m, p);
}

int lqt_mlp_get_params(lqt_mlp *m, float *params_host, float *grads_host)
{
    if (!m) return fail(LQT_ERR_INVALID, "lqt_mlp_get_params: NULL");
    CK(cudaStreamSynchronize(m->stream));
    if (params_host) CK(cudaMemcpy(params_host, m->P, kNParam * 4, cudaMemcpyDeviceToHost));
    if (grads_host) CK(cudaMemcpy(grads_host, m->G, kNParam * 4, cudaMemcpyDeviceToHost));
    return LQT_OK;
}

int lqt_mlp_set_norm(lqt_mlp *m, const float *in_mean, const float *in_scale, const float *out_scale, int32_t nvalid)
{
    if (!m || !in_mean || !in_scale || !out_scale || nvalid < 1 || nvalid > kMlpOut)
        return fail(LQT_ERR_INVALID, "lqt_mlp_set_norm: NULL or nvalid outside 1..48");
    std::vector<float> v(3 * kMlpIn);
    std::memcpy(v.data(), in_mean, kMlpIn * 4);
    std::memcpy(v.data() + kMlpIn, in_scale, kMlpIn * 4);
    std::memcpy(v.data() + 2 * kMlpIn, out_scale, kMlpOut * 4);
    CK(cudaMemcpy(m->norm, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
    m->nvalid = nvalid;
    return LQT_OK;
}

int lqt_mlp_set_bounds(lqt_mlp *m, const float *out_bound)
{
    if (!m || !out_bound) return fail(LQT_ERR_INVALID, "lqt_mlp_set_bounds: NULL");
    for (int i = 0; i < kMlpOut; ++i)
        if (!(out_bound[i] > 0)) return fail(LQT_ERR_INVALID, "lqt_mlp_set_bounds: bounds must be > 0");
    CK(cudaMemcpy(m->norm + 3 * kMlpIn, out_bound, kMlpOut * 4, cudaMemcpyHostToDevice));
    return LQT_OK;
}

int lqt_mlp_set_layout(lqt_mlp *m, int32_t layout)
{
    if (!m || (layout != 0 && layout != 1)) return fail(LQT_ERR_INVALID, "lqt_mlp_set_layout: 0 or 1");
    m->layout = layout;
    return LQT_OK;
}

int lqt_mlp_infer(lqt_mlp *m, const void *x_bf16_dev, float *y_dev, int64_t n)
{
    if (!m || !x_bf16_dev || !y_dev || n < 0) return fail(LQT_ERR_INVALID, "lqt_mlp_infer: NULL or n < 0");
    CK(cudaMemsetAsync(m->err, 0, 4, m->stream));
    CK(launch_mlp_infer_tc((const __nv_bfloat16 *)x_bf16_dev, y_dev, m->dev(), n, m->err, m->layout, m->stream));
    int err = 0;
    CK(cudaMemcpyAsync(&err, m->err, 4, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (err) return fail(LQT_ERR_TIMEOUT, "lqt_mlp_infer: tensor-core completion wait timed out");
    return LQT_OK;
}

int lqt_mlp_gradients(lqt_mlp *m, const void *x_bf16_dev, const float *t_dev, int64_t batch, double *loss)
{
    if (!m || !x_bf16_dev || !t_dev) return fail(LQT_ERR_INVALID, "lqt_mlp_gradients: NULL");
    int rc = forward_backward(m, (const __nv_bfloat16 *)x_bf16_dev, t_dev, batch);
    if (rc) return rc;
    double l = 0;
    int err = 0;
    CK(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(&err, m->err, 4, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (err) return fail(LQT_ERR_TIMEOUT, "lqt_mlp_gradients: tensor-core completion wait timed out");
    if (loss) *loss = l / ((double)batch * m->nvalid);
    return LQT_OK;
}

int lqt_mlp_train_step(lqt_mlp *m, const void *x_bf16_dev, const float *t_dev, int64_t batch, float lr, double *loss)
{
    if (!m || !x_bf16_dev || !t_dev || !(lr > 0)) return fail(LQT_ERR_INVALID, "lqt_mlp_train_step: NULL or lr <= 0");
    int rc = forward_backward(m, (const __nv_bfloat16 *)x_bf16_dev, t_dev, batch);
    if (rc) return rc;
    m->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
    CK(launch_adam(m->P, m->G, m->M, m->V, m->Pb, kNParam, lr, b1, b2, 1e-8f, c1, c2, m->stream));
    if (loss) {
        double l = 0;
        int err = 0;
        CK(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
        CK(cudaMemcpyAsync(&err, m->err, 4, cudaMemcpyDeviceToHost, m->stream));
        CK(cudaStreamSynchronize(m->stream));
        if (err) return fail(LQT_ERR_TIMEOUT, "lqt_mlp_train_step: tensor-core completion wait timed out");
        *loss = l / ((double)batch * m->nvalid);
    }
    return LQT_OK;
}

}  // extern "C"

// ---- training data ------------------------------------------------------------
#include "sur.h"

extern "C" {

int lqt_sur_datagen(int64_t ncells, uint64_t seed, const lqt_sur_ranges *r, float *x_dev, float *d_dev, int64_t cap,
                    int64_t *count, void *stream)
{
    if (ncells <= 0 || !r || !x_dev || !d_dev || cap <= 0 || !count)
        return fail(LQT_ERR_INVALID, "lqt_sur_datagen: bad arguments");
    if (!(r->bcl[0] > 10) || r->bcl[1] < r->bcl[0] || r->beats_warm < 0 || r->beats_record < 1 || !(r->dt > 0) ||
        !(r->prob > 0) || r->prob > 1 || !(r->jitter >= 0))
        return fail(LQT_ERR_INVALID, "lqt_sur_datagen: ranges (bcl > 10, beats_record >= 1, 0 < prob <= 1, dt > 0, jitter >= 0)");
    const int nsub = sur_nsub_or_default(r->nsub);
    if (!sur_nsub_ok(nsub) || r->reserved != 0)
        return fail(LQT_ERR_INVALID, "lqt_sur_datagen: nsub must divide 50 (0 = 5); reserved must be zero");
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<SurCell> cells(ncells);
    std::vector<ModelK> models(ncells);
    for (int64_t i = 0; i < ncells; ++i) {
        lqt_model mm{};
        mm.pca_scale = r->pca[0] + (r->pca[1] - r->pca[0]) * U(rng);
        mm.gks_scale = r->gks[0] + (r->gks[1] - r->gks[0]) * U(rng);
        mm.gks_iso_scale = r->iso[0] + (r->iso[1] - r->iso[0]) * U(rng);
        models[i] = make_modelk(mm);
        const double bcl = r->bcl[0] + (r->bcl[1] - r->bcl[0]) * U(rng);
        SurCell &c = cells[i];
        c.bcl_steps = (int64_t)std::llround(bcl / r->dt);
        c.warm_steps = c.bcl_steps * r->beats_warm;
        c.nsteps = c.bcl_steps * (r->beats_warm + r->beats_record);
        c.stim_on = (int64_t)std::llround(50.0 / r->dt);
        c.stim_off = c.stim_on + (int64_t)std::llround(2.0 / r->dt);
        c.model = (int32_t)i;
        const double u = U(rng);
        c.ctype = u < 1.0 / 3 ? LQT_ENDO : (u < 2.0 / 3 ? LQT_MCELL : LQT_EPI);
        c.stim = -52.f;
        c.gks_scale = (float)mm.gks_scale;
        c.pca_scale = (float)mm.pca_scale;
        c.iso_scale = (float)mm.gks_iso_scale;
    }
    DevMem tmp;
    SurCell *dc = nullptr;
    ModelK *dm = nullptr;
    int64_t *per_cell = nullptr;
    if (tmp.alloc((void **)&dc, ncells * sizeof(SurCell)) | tmp.alloc((void **)&dm, ncells * sizeof(ModelK)) |
        tmp.alloc((void **)&per_cell, ncells * sizeof(int64_t)))
        return LQT_ERR_NOMEM;
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(dc, cells.data(), ncells * sizeof(SurCell), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dm, models.data(), ncells * sizeof(ModelK), cudaMemcpyHostToDevice, st));
    // pass 1: pairs per cell; rows in cell order; pass 2: the pairs at their rows
    CK(launch_sur_datagen(dc, ncells, dm, make_stepk(r->dt), make_stepk(nsub * r->dt), nullptr, nullptr, per_cell,
                          nullptr, cap, seed, (float)r->dvdt_max, (float)r->prob, (float)r->jitter, nsub, st));
    std::vector<int64_t> off(ncells);
    CK(cudaMemcpyAsync(off.data(), per_cell, ncells * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int64_t total = 0;
    for (int64_t i = 0; i < ncells; ++i) {
        const int64_t c = off[i];
        off[i] = total;
        total += c;
    }
    CK(cudaMemcpyAsync(per_cell, off.data(), ncells * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CK(launch_sur_datagen(dc, ncells, dm, make_stepk(r->dt), make_stepk(nsub * r->dt), x_dev, d_dev, nullptr,
                          per_cell, cap, seed, (float)r->dvdt_max, (float)r->prob, (float)r->jitter, nsub, st));
    CK(cudaStreamSynchronize(st));
    *count = std::min<int64_t>(total, cap);
    return LQT_OK;
}

int lqt_sur_prepare(lqt_mlp *m, const float *x_dev, const float *d_dev, const int64_t *idx_dev, int64_t n,
                    void *xb_dev, float *t_dev)
{
    if (!m || !x_dev || !xb_dev || n < 0) return fail(LQT_ERR_INVALID, "lqt_sur_prepare: bad arguments");
    CK(launch_sur_prepare(x_dev, d_dev, idx_dev, n, m->norm, (__nv_bfloat16 *)xb_dev, d_dev ? t_dev : nullptr,
                          m->stream));
    return LQT_OK;
}

}  // extern "C"
