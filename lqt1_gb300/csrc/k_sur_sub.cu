// k_sur_sub.cu -- the V-only step of the voxels inside a surrogate macro step,
// mixed form, 1D/2D/3D: k_sur_substep (k_grid.cuh, one thread per voxel,
// direct loads) and k_sur_substep_tile (below, persistent CTAs that stage
// each tile's streamed rows in shared memory with bulk asynchronous copies).
#include <atomic>
#include <cstddef>

#include "k_grid.cuh"
#include "tc.cuh"

namespace lqt {

namespace {

constexpr uint32_t kSubWaitLimit = 1u << 22;   // bounded mbarrier polls per tile

// One tile's rows, in the order of the copies: the macro step's ionic rate,
// the dense index, the FP16 tensor row (3 half2 per voxel: the scaled fibre
// direction and the divergence, GridDev::t3h), the control byte and the
// detector flag.
struct __align__(16) SubStage {
    float rate[kSubTile];
    int32_t gidx[kSubTile];
    __half2 t3[kSubTile * 3];
    uint8_t ctl[kSubTile];
    uint8_t flag[kSubTile];
};
static_assert(sizeof(SubStage) % 16 == 0 && offsetof(SubStage, gidx) % 16 == 0 && offsetof(SubStage, t3) % 16 == 0 &&
                  offsetof(SubStage, ctl) % 16 == 0 && offsetof(SubStage, flag) % 16 == 0,
              "bulk copies need 16-byte aligned destinations");

// Thread 0: the copies of tile k0 / kSubTile into one stage, completing on bar.
// Every array holds whole tiles (pad_tiles), so each copy is in bounds, and
// k0 is a multiple of kSubTile, so every source is 16-byte aligned.
__device__ __forceinline__ void sub_issue(SubStage &sg, uint64_t *bar, const GridDev<float> &gd, int64_t k0, bool det)
{
    constexpr uint32_t n = kSubTile;
    tc::mbar_expect_tx(bar, n * (4 + 4 + 12 + 1) + (det ? n : 0));
    tc::bulk_g2s(sg.rate, gd.srate + k0, n * 4, bar);
    tc::bulk_g2s(sg.gidx, gd.gidx + k0, n * 4, bar);
    tc::bulk_g2s(sg.t3, gd.t3h + 3 * k0, n * 12, bar);
    tc::bulk_g2s(sg.ctl, gd.ctl + k0, n, bar);
    if (det) tc::bulk_g2s(sg.flag, gd.sdflag + k0, n, bar);
}

}  // namespace

// Persistent: CTA b takes tiles b, b + gridDim.x, ...  Two stages: while the
// threads step the voxels of one tile (V stencil from the dense grid, through
// L1/L2), the copy engine brings the next tile's rows, so the streamed bytes
// stay in flight without a per-thread load chain in front of the stencil.
// Arithmetic identical to k_sur_substep.  A copy wait that runs out sets bit 1
// of *serr; the CTA waits (bounded) for its copies still in flight and leaves
// its remaining tiles unstepped.  gd.sub_skip_copy / gd.sub_wait_limit drive
// that path in a test: the first tile's copies are left out and the wait
// bound shortened, so the wait runs out on a phase nothing completes.
template <int DIM, int MINB>
__global__ void __launch_bounds__(kSubTile, MINB) k_sur_substep_tile(GridDev<float> gd, float dt, int cur)
{
    __shared__ SubStage stg[2];
    __shared__ __align__(8) uint64_t bar[2];
    const int t = threadIdx.x;
    const int64_t ntiles = (gd.ntissue + kSubTile - 1) / kSubTile;
    const int64_t stride = gridDim.x;
    int64_t tile = blockIdx.x;
    if (tile >= ntiles) return;
    const bool det = gd.det != nullptr;
    const uint32_t lim = gd.sub_wait_limit ? gd.sub_wait_limit : kSubWaitLimit;
    if (t == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // (a failure-path test leaves the first tile's copies out: nothing
        // completes that phase and its wait runs out)
        if (!gd.sub_skip_copy) sub_issue(stg[0], &bar[0], gd, tile * kSubTile, det);
        if (tile + stride < ntiles) sub_issue(stg[1], &bar[1], gd, (tile + stride) * kSubTile, det);
    }
    __syncthreads();
    const Clock ck = *gd.clk;
    const float *__restrict__ V = gd.vg[cur];
    float *__restrict__ Vn = gd.vg[cur ^ 1];
    for (uint32_t it = 0; tile < ntiles; tile += stride, ++it) {
        const int s = it & 1;
        const bool ok = tc::mbar_wait(&bar[s], (it >> 1) & 1, lim);
        if (!__syncthreads_and(ok ? 1 : 0)) {
            if (t == 0) {
                atomicOr(gd.serr, 2);
                // let this CTA's copies in flight land before it leaves
                // (the full bound: these are real copies; a first tile left
                // out by the failure-path test has none)
                if (it > 0 || !gd.sub_skip_copy) tc::mbar_wait(&bar[s], (it >> 1) & 1, kSubWaitLimit);
                if (tile + stride < ntiles) tc::mbar_wait(&bar[s ^ 1], ((it + 1) >> 1) & 1, kSubWaitLimit);
            }
            return;
        }
        const SubStage &sg = stg[s];
        const int64_t k = tile * kSubTile + t;
        const float r = sg.rate[t];
        if (k < gd.ntissue && r == r) {
            const int64_t g = sg.gidx[t];
            float2 q[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) q[i] = __half22float2(sg.t3[3 * t + i]);
            float Dt[6], Bt[3];
            sub_tensor_unpack<DIM>(q, gd.sub_dtr, gd.sub_dsg, Dt, Bt);
            const float vc = V[g];
            const float du = sub_du<DIM>(gd, V, g, k, vc, Dt, Bt);
            const float ist = grid_stim(gd, ck, sg.ctl[t], k);
            const float dvdt = r - ist;
            const float vn = vc + (dvdt + du) * dt;
            Vn[g] = vn;
            if (det && sg.flag[t]) grid_detect(gd, ck, k, vc, vn, dvdt);
            const bool bad = !(vn == vn) || vn < gd.vmin_ok || vn > gd.vmax_ok;
            if (bad) atomicAdd(gd.nbad, 1ull);
        }
        __syncthreads();   // every thread is done with stage s
        if (t == 0 && tile + 2 * stride < ntiles) {
            tc::fence_proxy_async();
            sub_issue(stg[s], &bar[s], gd, (tile + 2 * stride) * kSubTile, det);
        }
    }
}

namespace {

// One stage of the V-halo kernel: the tile's streamed rows, each voxel's index
// in the tile's V box, the box itself and the tile's box header.
struct __align__(16) VStage {
    SubStage rows;
    int32_t li[kSubTile];
    float vb[kVBoxFloats];
    int32_t hdr[8];
};
static_assert(offsetof(VStage, li) % 16 == 0 && offsetof(VStage, vb) % 16 == 0 && sizeof(VStage) % 16 == 0,
              "bulk copies need 16-byte aligned destinations");
// The rows-only stage of the same pipeline (no V box).
struct __align__(16) RStage {
    SubStage rows;
    int32_t hdr[8];
};
template <bool BOX> struct StageOf { using T = VStage; };
template <> struct StageOf<false> { using T = RStage; };

struct VHdr {
    int32_t ok, zlo, xlo, ylo, bx, by, bz;
};

__device__ __forceinline__ VHdr vhdr_load(const int32_t *h)
{
    const int4 a = __ldg(reinterpret_cast<const int4 *>(h)), b = __ldg(reinterpret_cast<const int4 *>(h) + 1);
    return VHdr{a.x, a.y, a.z, a.w, b.x, b.y, b.z};
}

// The producer warp's share of the copies of tile k0 / kSubTile into one
// stage: lane 0 first writes the header and arms the stage's mbarrier with
// the byte count, then the lanes issue the copies in parallel -- the 6 row
// copies (rate, index, tensor row, control, detector flag, box index; 5
// without the box) and, when the box fits, one per box column.  A box column is the
// z-segment [zlo, zlo + bz) of grid column (xlo + i, ylo + j), copied whole:
// nz, zlo and bz are multiples of 4, so every source and destination is
// 16-byte aligned and every size a multiple of 16 bytes; the host builder
// keeps every segment inside its column and every column inside the grid.
template <bool BOX>
__device__ __forceinline__ void vbox_issue(typename StageOf<BOX>::T &st, uint64_t *bar, const GridDev<float> &gd,
                                           const float *V, int64_t k0, bool det, const VHdr &h, int lane, int64_t ny,
                                           int64_t nz)
{
    constexpr uint32_t n = kSubTile;
    const int ncol = (BOX && h.ok) ? h.bx * h.by : 0;
    if (lane == 0) {
        st.hdr[0] = BOX ? h.ok : 0;
        st.hdr[1] = h.by * h.bz;
        st.hdr[2] = h.bz;
        const uint32_t box = (uint32_t)ncol * (uint32_t)h.bz * 4u;
        tc::mbar_expect_tx(bar, n * (4 + 4 + 12 + 1) + (det ? n : 0) + (BOX ? n * 4 : 0) + box);
    }
    __syncwarp();
    for (int c = lane; c < (BOX ? 6 : 5) + ncol; c += 32) {
        switch (c) {
        case 0: tc::bulk_g2s(st.rows.rate, gd.srate + k0, n * 4, bar); break;
        case 1: tc::bulk_g2s(st.rows.gidx, gd.gidx + k0, n * 4, bar); break;
        case 2: tc::bulk_g2s(st.rows.t3, gd.t3h + 3 * k0, n * 12, bar); break;
        case 3: tc::bulk_g2s(st.rows.ctl, gd.ctl + k0, n, bar); break;
        case 4: if (det) tc::bulk_g2s(st.rows.flag, gd.sdflag + k0, n, bar); break;
        default:
            if constexpr (BOX) {
                if (c == 5) {
                    tc::bulk_g2s(st.li, gd.vli + k0, n * 4, bar);
                } else {
                    const int col = c - 6, i = col / h.by, j = col - i * h.by;
                    tc::bulk_g2s(st.vb + col * h.bz, V + ((int64_t)(h.xlo + i) * ny + (h.ylo + j)) * nz + h.zlo,
                                 (uint32_t)h.bz * 4u, bar);
                }
            }
        }
    }
}

// Named barrier over the 256 consumer threads (id 1) that also returns
// whether every one of them passed `v` != 0.
__device__ __forceinline__ int consumers_and(int v)
{
    int r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.and.pred q, 1, %2, p;\nselp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(v), "n"(kSubTile)
        : "memory");
    return r;
}

}  // namespace

// 3D V-only substep with the V halo staged.  Persistent CTAs of 8 consumer
// warps (one voxel per thread of a 256-voxel tile) and one producer warp, two
// stages: each stage holds a tile's streamed rows and the box of the dense V
// grid its stencils reach.  The producer fills a stage as soon as the
// consumers release it (mbarrier `empty`) and arms `full` with the stage's
// byte count; the consumers wait on `full`, read the 19-point stencil from
// shared memory and release the stage -- no CTA-wide barrier per tile.  A
// tile whose box exceeds the stage reads V from the grid.  Arithmetic
// identical to k_sur_substep.  Every wait is bounded: a consumer wait that
// runs out sets bit 1 of *serr and ends the consumers' loop; a producer wait
// that runs out stops the issuing; before leaving, the producer waits
// (bounded) until the copies it issued have landed.  With BOX false the
// stages hold the rows only and V comes from the grid (2D and 3D).
template <int DIM, int MINB, bool BOX>
__global__ void __launch_bounds__(kSubTile + 32, MINB) k_sur_substep_vbox(GridDev<float> gd, float dt, int cur)
{
    using Stage = typename StageOf<BOX>::T;
    extern __shared__ __align__(128) uint8_t vsm[];
    Stage *stg = reinterpret_cast<Stage *>(vsm);
    __shared__ __align__(8) uint64_t full[2], empty[2];
    const int t = threadIdx.x;
    const int64_t ntiles = (gd.ntissue + kSubTile - 1) / kSubTile;
    const int64_t stride = gridDim.x;
    const int64_t tile0 = blockIdx.x;
    if (tile0 >= ntiles) return;
    const bool det = gd.det != nullptr;
    const uint32_t lim = gd.sub_wait_limit ? gd.sub_wait_limit : kSubWaitLimit;
    const float *__restrict__ V = gd.vg[cur];
    if (t == 0) {
        tc::mbar_init(&full[0], 1);
        tc::mbar_init(&full[1], 1);
        tc::mbar_init(&empty[0], kSubTile / 32);
        tc::mbar_init(&empty[1], kSubTile / 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (t >= kSubTile) {
        // ---- producer warp ----
        const int lane = t - kSubTile;
        const int64_t ny = BOX ? gd.sx / gd.sy : 0, nz = BOX ? gd.sy : 0;
        const bool skip0 = gd.sub_skip_copy != 0;   // failure-path test: tile 0's stage is never filled
        uint32_t issued = 0;
        for (int64_t tile = tile0; tile < ntiles; tile += stride, ++issued) {
            const int s = issued & 1;
            // the whole warp takes one decision (vbox_issue synchronises the warp)
            const bool free = issued < 2 || tc::mbar_wait(&empty[s], ((issued - 2) >> 1) & 1, lim);
            if (!__all_sync(0xffffffffu, free)) {
                if (lane == 0) atomicOr(gd.serr, 2);
                break;
            }
            if (issued == 0 && skip0) continue;
            tc::fence_proxy_async();
            const VHdr h = BOX ? vhdr_load(gd.vbox_hdr + 8 * tile) : VHdr{};
            vbox_issue<BOX>(stg[s], &full[s], gd, V, tile * kSubTile, det, h, lane, ny, nz);
        }
        // the copies of the last two stages have landed before the CTA ends
        for (uint32_t j = issued > 2 ? issued - 2 : 0; j < issued; ++j)
            if (j > 0 || !skip0) tc::mbar_wait(&full[j & 1], (j >> 1) & 1, kSubWaitLimit);
        return;
    }
    // ---- consumer warps ----
    float *__restrict__ Vn = gd.vg[cur ^ 1];
    const Clock ck = *gd.clk;
    uint32_t it = 0;
    for (int64_t tile = tile0; tile < ntiles; tile += stride, ++it) {
        const int s = it & 1;
        const bool ok = tc::mbar_wait(&full[s], (it >> 1) & 1, lim);
        if (!consumers_and(ok ? 1 : 0)) {
            if (t == 0) atomicOr(gd.serr, 2);
            break;
        }
        const Stage &st = stg[s];
        const SubStage &sg = st.rows;
        const int64_t k = tile * kSubTile + t;
        const float r = sg.rate[t];
        if (k < gd.ntissue && r == r) {
            const int64_t g = sg.gidx[t];
            float2 q[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) q[i] = __half22float2(sg.t3[3 * t + i]);
            float Dt[6], Bt[3];
            sub_tensor_unpack<DIM>(q, gd.sub_dtr, gd.sub_dsg, Dt, Bt);
            float vc, du;
            bool staged = false;
            if constexpr (BOX) {
                if (st.hdr[0]) {
                    const int64_t li = st.li[t];
                    vc = st.vb[li];
                    du = sub_du_at<DIM>(gd, st.vb, li, st.hdr[1], st.hdr[2], vc, Dt, Bt);
                    staged = true;
                }
            }
            if (!staged) {
                vc = V[g];
                du = sub_du_at<DIM>(gd, V, g, gd.sx, gd.sy, vc, Dt, Bt);
            }
            const float ist = grid_stim(gd, ck, sg.ctl[t], k);
            const float dvdt = r - ist;
            const float vn = vc + (dvdt + du) * dt;
            Vn[g] = vn;
            if (det && sg.flag[t]) grid_detect(gd, ck, k, vc, vn, dvdt);
            const bool bad = !(vn == vn) || vn < gd.vmin_ok || vn > gd.vmax_ok;
            if (bad) atomicAdd(gd.nbad, 1ull);
        }
        __syncwarp();
        if ((t & 31) == 0) tc::mbar_arrive(&empty[s]);   // this warp is done with stage s
    }
}

namespace {

template <int MINB> void launch_minb(const GridDev<float> &gd, double dt, int cur, int dim, unsigned nb, cudaStream_t st)
{
    if (dim == 1) k_sur_substep<1, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else if (dim == 2) k_sur_substep<2, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else k_sur_substep<3, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
}

// The kernel's shared-memory carve-out at its maximum, once per device, so
// that MINB CTAs of two stages each fit on an SM.
template <typename K> cudaError_t carveout_once(K kernel, std::atomic<uint64_t> &done)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0;
    if (bit && (done.load() & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess && bit) done.fetch_or(bit);
    return e;
}

template <int DIM, int MINB> cudaError_t launch_tile(const GridDev<float> &gd, double dt, int cur, cudaStream_t st)
{
    static std::atomic<uint64_t> done{0};
    cudaError_t e = carveout_once(k_sur_substep_tile<DIM, MINB>, done);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t ntiles = (gd.ntissue + kSubTile - 1) / kSubTile;
    const int64_t grid = ntiles < (int64_t)nsm * MINB ? ntiles : (int64_t)nsm * MINB;
    k_sur_substep_tile<DIM, MINB><<<(unsigned)grid, kSubTile, 0, st>>>(gd, (float)dt, cur);
    return cudaGetLastError();
}

template <int DIM, int MINB, bool BOX>
cudaError_t launch_vbox(const GridDev<float> &gd, double dt, int cur, cudaStream_t st)
{
    static std::atomic<uint64_t> done{0}, carve{0};
    const uint32_t bytes = 2 * sizeof(typename StageOf<BOX>::T);
    cudaError_t e = tc::smem_attr_once(k_sur_substep_vbox<DIM, MINB, BOX>, bytes, done);
    if (e == cudaSuccess) e = carveout_once(k_sur_substep_vbox<DIM, MINB, BOX>, carve);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t ntiles = (gd.ntissue + kSubTile - 1) / kSubTile;
    const int64_t grid = ntiles < (int64_t)nsm * MINB ? ntiles : (int64_t)nsm * MINB;
    k_sur_substep_vbox<DIM, MINB, BOX><<<(unsigned)grid, kSubTile + 32, bytes, st>>>(gd, (float)dt, cur);
    return cudaGetLastError();
}

bool al16(const void *p) { return p && ((uintptr_t)p & 15u) == 0; }

}  // namespace

cudaError_t launch_sur_substep(const GridDev<float> &gd, double dt, int cur, int dim, int variant, cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    const bool rows_ok = dim >= 2 && gd.d6 && al16(gd.t3h) && al16(gd.srate) && al16(gd.gidx) &&
                         al16(gd.ctl) && gd.serr && (!gd.det || al16(gd.sdflag));
    if (variant >= 300) {
        // rows staged by a producer warp, V from the grid (2D/3D)
        if (rows_ok) {
            if (dim == 2) {
                if (variant == 306) return launch_vbox<2, 6, false>(gd, dt, cur, st);
                if (variant == 305) return launch_vbox<2, 5, false>(gd, dt, cur, st);
                return launch_vbox<2, 4, false>(gd, dt, cur, st);
            }
            if (variant == 306) return launch_vbox<3, 6, false>(gd, dt, cur, st);
            if (variant == 305) return launch_vbox<3, 5, false>(gd, dt, cur, st);
            return launch_vbox<3, 4, false>(gd, dt, cur, st);
        }
        variant = 105;
    } else if (variant >= 200) {
        if (dim == 3 && rows_ok && gd.vbox_hdr && gd.vli && al16(gd.vli) && al16(gd.vg[0]) && al16(gd.vg[1]))
            return variant == 203 ? launch_vbox<3, 3, true>(gd, dt, cur, st) : launch_vbox<3, 4, true>(gd, dt, cur, st);
        variant = 105;
    }
    const bool tile = variant >= 100;
    const int minb = tile ? variant - 100 : variant;
    if (dim >= 2 && gd.d6 && !gd.t3h) return cudaErrorInvalidValue;   // FP16 tensor rows missing
    if (tile && dim >= 2 && gd.d6 && al16(gd.t3h) && al16(gd.srate) && al16(gd.gidx) &&
        al16(gd.ctl) && gd.serr && (!gd.det || al16(gd.sdflag))) {
        if (dim == 2) {
            if (minb == 8) return launch_tile<2, 8>(gd, dt, cur, st);
            if (minb == 6) return launch_tile<2, 6>(gd, dt, cur, st);
            return launch_tile<2, 5>(gd, dt, cur, st);
        }
        if (minb == 8) return launch_tile<3, 8>(gd, dt, cur, st);
        if (minb == 6) return launch_tile<3, 6>(gd, dt, cur, st);
        return launch_tile<3, 5>(gd, dt, cur, st);
    }
    const unsigned nb = (unsigned)((gd.ntissue + 256 * kSubU - 1) / (256 * kSubU));
    if (minb == 8) launch_minb<8>(gd, dt, cur, dim, nb, st);
    else if (minb == 6) launch_minb<6>(gd, dt, cur, dim, nb, st);
    else launch_minb<5>(gd, dt, cur, dim, nb, st);
    return cudaGetLastError();
}

}  // namespace lqt
