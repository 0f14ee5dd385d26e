// k_geom.cu -- tissue numbering and the mirror-boundary map built on the GPU.
//
// The reference builds both on the host before every 2D/3D run
// (GPU3D.cu:1307-1333 numbering, 1487-1604 mirror map; new_11.cu:1535-1640):
// a pass over every grid voxel that, for each empty voxel with a tissue
// neighbour, estimates an outward normal from the weighted occupancy of its
// neighbours and picks the tissue neighbour nearest to that direction.  Here
// the same search runs one thread per grid voxel:
//   1. k_geom_count: per block of kVoxPerBlock consecutive voxels, the number
//      of tissue voxels and of boundary voxels (empty, with a tissue
//      neighbour);
//   2. k_geom_scan: one CTA turns the block counts into exclusive offsets;
//   3. k_geom_emit: every voxel's tissue index (or -1), the tissue list, and
//      for boundary voxels the mirror source, written in grid order.
// The result is the host builder's (geometry.cc) bit for bit: the normal's
// FP64 sums take the terms in the reference's order and every operation is
// written as an explicitly rounded IEEE operation (no FMA contraction), so
// ties in the nearest-voxel search break the same way.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lqt.h"
#include "api_common.h"
#include "geometry.h"
#include "mirror_tables.h"

namespace lqt {

namespace {

constexpr int kGeoThreads = 256;
constexpr int kVoxPerThread = 16;
constexpr int kVoxPerBlock = kGeoThreads * kVoxPerThread;

__constant__ int8_t c_ic3[18][3] = LQT_MIRROR_IC3;
__constant__ int8_t c_ir3[18][3] = LQT_MIRROR_IR3;
__constant__ int8_t c_il3[18][3] = LQT_MIRROR_IL3;
__constant__ int8_t c_il2[6][3] = LQT_MIRROR_IL2;
__constant__ int8_t c_ir2[6][3] = LQT_MIRROR_IR2;
__constant__ int c_slot2x[9] = LQT_MIRROR_SLOT2X;
__constant__ int c_slot2y[9] = LQT_MIRROR_SLOT2Y;

struct GeoDims {
    int64_t nx, ny, nz, total;
};

__device__ __forceinline__ bool is_tissue(const uint8_t *__restrict__ t, const GeoDims &d, int64_t x, int64_t y,
                                          int64_t z)
{
    return x >= 0 && x < d.nx && y >= 0 && y < d.ny && z >= 0 && z < d.nz && t[(x * d.ny + y) * d.nz + z] != LQT_EMPTY;
}

// Occupancy of the 26 (3D) or 8 (2D) neighbours of an empty voxel, in slot
// order; returns the number of tissue neighbours.
__device__ __forceinline__ int neighbours(const uint8_t *__restrict__ t, const GeoDims &d, int64_t x, int64_t y,
                                          int64_t z, int *gg)
{
    int nb = 0;
    gg[0] = 0;
    if (d.nz == 1) {
        for (int k = 1; k <= 8; ++k) {
            gg[k] = is_tissue(t, d, x + c_slot2x[k], y + c_slot2y[k], 0);
            nb += gg[k];
        }
    } else {
        int k = 0;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    if (!ox && !oy && !oz) continue;
                    gg[++k] = is_tissue(t, d, x + ox, y + oy, z + oz);
                    nb += gg[k];
                }
    }
    return nb;
}

// One component of the normal: the terms in table order, each g, g/sqrt2 or
// g/sqrt3, added or subtracted in FP64 with IEEE rounding.
__device__ __forceinline__ double occ_sum(const int8_t (*tab)[3], int n, const int *gg)
{
    const double r2 = __dsqrt_rn(2.0), r3 = __dsqrt_rn(3.0);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
        const double g = (double)gg[tab[i][0]];
        const double term = tab[i][1] == 1 ? g : __ddiv_rn(g, tab[i][1] == 2 ? r2 : r3);
        acc = tab[i][2] > 0 ? __dadd_rn(acc, term) : __dsub_rn(acc, term);
    }
    return acc;
}

// The mirror source of boundary voxel (x, y, z): the tissue neighbour nearest
// to the estimated outward normal (first strict minimum in z, y, x order).
__device__ int64_t mirror_source(const uint8_t *__restrict__ t, const GeoDims &d, int64_t x, int64_t y, int64_t z,
                                 const int *gg)
{
    const bool is2d = d.nz == 1;
    double il, ir, ic = 0.0, imax;
    if (is2d) {
        il = occ_sum(c_il2, 6, gg);
        ir = occ_sum(c_ir2, 6, gg);
        imax = fabs(il);
        if (fabs(ir) > imax) imax = fabs(ir);
    } else {
        ic = occ_sum(c_ic3, 18, gg);
        ir = occ_sum(c_ir3, 18, gg);
        il = occ_sum(c_il3, 18, gg);
        imax = fabs(ic);
        if (fabs(ir) > imax) imax = fabs(ir);
        if (fabs(il) > imax) imax = fabs(il);
    }
    double nxv = __ddiv_rn(il, imax), nyv = __ddiv_rn(ir, imax), nzv = is2d ? 0.0 : __ddiv_rn(ic, imax);
    if (__dsub_rn(imax, 0.0) < 0.0001) nxv = nyv = nzv = 0.0;
    double best = 1000;
    int bx = 0, by = 0, bz = 0;
    const int zlo = is2d ? 0 : -1, zhi = is2d ? 0 : 1;
    for (int zc = zlo; zc <= zhi; ++zc)
        for (int yc = -1; yc <= 1; ++yc)
            for (int xc = -1; xc <= 1; ++xc) {
                const double a = __dsub_rn((double)xc, nxv), b = __dsub_rn((double)yc, nyv);
                double s = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
                if (!is2d) {
                    const double c = __dsub_rn((double)zc, nzv);
                    s = __dadd_rn(s, __dmul_rn(c, c));
                }
                const double dis = __dsqrt_rn(s);
                if (is_tissue(t, d, x + xc, y + yc, z + zc) && dis < best) {
                    bx = xc;
                    by = yc;
                    bz = zc;
                    best = dis;
                }
            }
    return ((x + bx) * d.ny + (y + by)) * d.nz + (z + bz);
}

// Kind of grid voxel g: 1 tissue, 2 boundary (empty with a tissue neighbour), 0 other.
__device__ __forceinline__ int voxel_kind(const uint8_t *__restrict__ t, const GeoDims &d, int64_t g, int *gg)
{
    if (t[g] != LQT_EMPTY) return 1;
    const int64_t x = g / (d.ny * d.nz), r = g - x * d.ny * d.nz, y = r / d.nz, z = r - y * d.nz;
    return neighbours(t, d, x, y, z, gg) > 0 ? 2 : 0;
}

// Exclusive scan of one value per thread over the block (two counters packed
// as 32-bit halves of a 64-bit word: each is at most kVoxPerBlock).
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t *total)
{
    __shared__ uint64_t warp_sums[kGeoThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_sums[w] = inc;
    __syncthreads();
    uint64_t off = 0, tot = 0;
    for (int i = 0; i < kGeoThreads / 32; ++i) {
        if (i < w) off += warp_sums[i];
        tot += warp_sums[i];
    }
    __syncthreads();
    *total = tot;
    return off + inc - v;
}

__global__ void __launch_bounds__(kGeoThreads) k_geom_count(const uint8_t *__restrict__ t, GeoDims d,
                                                            int64_t *__restrict__ nt_blk, int64_t *__restrict__ nb_blk)
{
    const int64_t g0 = (int64_t)blockIdx.x * kVoxPerBlock + (int64_t)threadIdx.x * kVoxPerThread;
    uint64_t cnt = 0;
    int gg[27];
    for (int i = 0; i < kVoxPerThread; ++i) {
        const int64_t g = g0 + i;
        if (g >= d.total) break;
        const int k = voxel_kind(t, d, g, gg);
        cnt += k == 1 ? 1ull : (k == 2 ? (1ull << 32) : 0ull);
    }
    uint64_t tot;
    block_exclusive_scan(cnt, &tot);
    if (threadIdx.x == 0) {
        nt_blk[blockIdx.x] = (int64_t)(tot & 0xffffffffull);
        nb_blk[blockIdx.x] = (int64_t)(tot >> 32);
    }
}

// In-place exclusive scan of the block counts (one CTA); totals in tot[0..1].
__global__ void __launch_bounds__(1024) k_geom_scan(int64_t *__restrict__ nt_blk, int64_t *__restrict__ nb_blk,
                                                    int64_t nblk, int64_t *__restrict__ tot)
{
    __shared__ int64_t s_t[1024], s_b[1024];
    __shared__ int64_t carry_t, carry_b;
    if (threadIdx.x == 0) carry_t = carry_b = 0;
    __syncthreads();
    for (int64_t base = 0; base < nblk; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int64_t vt = i < nblk ? nt_blk[i] : 0, vb = i < nblk ? nb_blk[i] : 0;
        s_t[threadIdx.x] = vt;
        s_b[threadIdx.x] = vb;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {        // Hillis-Steele inclusive scan
            const int64_t at = threadIdx.x >= o ? s_t[threadIdx.x - o] : 0;
            const int64_t ab = threadIdx.x >= o ? s_b[threadIdx.x - o] : 0;
            __syncthreads();
            s_t[threadIdx.x] += at;
            s_b[threadIdx.x] += ab;
            __syncthreads();
        }
        if (i < nblk) {
            nt_blk[i] = carry_t + s_t[threadIdx.x] - vt;
            nb_blk[i] = carry_b + s_b[threadIdx.x] - vb;
        }
        __syncthreads();
        if (threadIdx.x == 1023) {
            carry_t += s_t[1023];
            carry_b += s_b[1023];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        tot[0] = carry_t;
        tot[1] = carry_b;
    }
}

__global__ void __launch_bounds__(kGeoThreads) k_geom_emit(const uint8_t *__restrict__ t, GeoDims d,
                                                           const int64_t *__restrict__ nt_off,
                                                           const int64_t *__restrict__ nb_off,
                                                           int32_t *__restrict__ tissue_of, int32_t *__restrict__ cells,
                                                           int32_t *__restrict__ bnd_dst, int32_t *__restrict__ bnd_src)
{
    const int64_t g0 = (int64_t)blockIdx.x * kVoxPerBlock + (int64_t)threadIdx.x * kVoxPerThread;
    int gg[27];
    uint64_t cnt = 0;
    for (int i = 0; i < kVoxPerThread; ++i) {
        const int64_t g = g0 + i;
        if (g >= d.total) break;
        const int k = voxel_kind(t, d, g, gg);
        cnt += k == 1 ? 1ull : (k == 2 ? (1ull << 32) : 0ull);
    }
    uint64_t tot;
    const uint64_t off = block_exclusive_scan(cnt, &tot);
    int64_t it = nt_off[blockIdx.x] + (int64_t)(off & 0xffffffffull);
    int64_t ib = nb_off[blockIdx.x] + (int64_t)(off >> 32);
    for (int i = 0; i < kVoxPerThread; ++i) {
        const int64_t g = g0 + i;
        if (g >= d.total) break;
        const int k = voxel_kind(t, d, g, gg);
        if (tissue_of) tissue_of[g] = k == 1 ? (int32_t)it : -1;
        if (k == 1) {
            if (cells) cells[it] = (int32_t)g;
            ++it;
        } else if (k == 2) {
            if (bnd_dst) {
                const int64_t x = g / (d.ny * d.nz), r = g - x * d.ny * d.nz, y = r / d.nz, z = r - y * d.nz;
                bnd_dst[ib] = (int32_t)g;
                bnd_src[ib] = (int32_t)mirror_source(t, d, x, y, z, gg);
            }
            ++ib;
        }
    }
}

}  // namespace

int64_t geom_map_blocks(int64_t total) { return (total + kVoxPerBlock - 1) / kVoxPerBlock; }

// Counts (tot_dev[0] tissue, [1] boundary) and offsets; scratch holds 2 x
// geom_map_blocks(total) int64.
cudaError_t launch_geom_count(const uint8_t *types_dev, int32_t nx, int32_t ny, int32_t nz, int64_t *scratch,
                              int64_t *tot_dev, cudaStream_t st)
{
    const GeoDims d{nx, ny, nz, (int64_t)nx * ny * nz};
    const int64_t nblk = geom_map_blocks(d.total);
    k_geom_count<<<(unsigned)nblk, kGeoThreads, 0, st>>>(types_dev, d, scratch, scratch + nblk);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_geom_scan<<<1, 1024, 0, st>>>(scratch, scratch + nblk, nblk, tot_dev);
    return cudaGetLastError();
}

// Outputs sized by the counts of launch_geom_count (any may be NULL except
// that bnd_dst and bnd_src go together).
cudaError_t launch_geom_emit(const uint8_t *types_dev, int32_t nx, int32_t ny, int32_t nz, const int64_t *scratch,
                             int32_t *tissue_of, int32_t *cells, int32_t *bnd_dst, int32_t *bnd_src, cudaStream_t st)
{
    const GeoDims d{nx, ny, nz, (int64_t)nx * ny * nz};
    const int64_t nblk = geom_map_blocks(d.total);
    k_geom_emit<<<(unsigned)nblk, kGeoThreads, 0, st>>>(types_dev, d, scratch, scratch + nblk, tissue_of, cells,
                                                        bnd_dst, bnd_src);
    return cudaGetLastError();
}

// The tissue map of a host grid, built on the current device: numbering,
// tissue list and mirror-boundary map, downloaded into `out` (the host
// builder's structure and order).  Device buffers live for the call only.
int build_tissue_map_gpu(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types_host, cudaStream_t st,
                         TissueMap &out)
{
    const int64_t total = (int64_t)nx * ny * nz;
    if (nx < 1 || ny < 1 || nz < 1 || total > (int64_t)INT32_MAX || !types_host)
        return fail(LQT_ERR_INVALID, "build_tissue_map_gpu: grid must be 1..2^31-1 voxels");
    const int64_t nblk = geom_map_blocks(total);
    DevMem mem;
    uint8_t *t_dev = nullptr;
    int64_t *scratch = nullptr, *tot_dev = nullptr;
    int32_t *tissue_of = nullptr;
    int rc = mem.alloc((void **)&t_dev, total) | mem.alloc((void **)&scratch, 2 * nblk * 8) |
             mem.alloc((void **)&tot_dev, 16) | mem.alloc((void **)&tissue_of, total * 4);
    if (rc) return fail(LQT_ERR_NOMEM, "build_tissue_map_gpu: device allocation failed: " + g_err);
    int64_t tot[2] = {0, 0};
    cudaError_t e = cudaMemcpyAsync(t_dev, types_host, total, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_geom_count(t_dev, nx, ny, nz, scratch, tot_dev, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tot, tot_dev, 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("build_tissue_map_gpu: ") + cudaGetErrorString(e));
    int32_t *cells = nullptr, *bd = nullptr, *bs = nullptr;
    rc = mem.alloc((void **)&cells, std::max<int64_t>(1, tot[0]) * 4) |
         mem.alloc((void **)&bd, std::max<int64_t>(1, tot[1]) * 4) |
         mem.alloc((void **)&bs, std::max<int64_t>(1, tot[1]) * 4);
    if (rc) return fail(LQT_ERR_NOMEM, "build_tissue_map_gpu: device allocation failed: " + g_err);
    std::vector<int32_t> cells_h((size_t)tot[0]), bd_h((size_t)tot[1]), bs_h((size_t)tot[1]);
    out.tissue_of.resize((size_t)total);
    e = launch_geom_emit(t_dev, nx, ny, nz, scratch, tissue_of, cells, bd, bs, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.tissue_of.data(), tissue_of, total * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && tot[0])
        e = cudaMemcpyAsync(cells_h.data(), cells, tot[0] * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && tot[1]) e = cudaMemcpyAsync(bd_h.data(), bd, tot[1] * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && tot[1]) e = cudaMemcpyAsync(bs_h.data(), bs, tot[1] * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(LQT_ERR_CUDA, std::string("build_tissue_map_gpu: ") + cudaGetErrorString(e));
    out.cells.assign(cells_h.begin(), cells_h.end());
    out.bnd_dst.assign(bd_h.begin(), bd_h.end());
    out.bnd_src.assign(bs_h.begin(), bs_h.end());
    return LQT_OK;
}

}  // namespace lqt

extern "C" int lqt_geom_mirror_map_gpu(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types, int32_t *tissue_of,
                                       int64_t *bnd_dst, int64_t *bnd_src, int64_t *nbnd, void *stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || !types || !nbnd)
        return lqt::fail(LQT_ERR_INVALID, "lqt_geom_mirror_map_gpu: bad arguments");
    lqt::TissueMap tm;
    const int rc = lqt::build_tissue_map_gpu(nx, ny, nz, types, (cudaStream_t)stream, tm);
    if (rc) return rc;
    *nbnd = (int64_t)tm.bnd_dst.size();
    if (tissue_of) std::memcpy(tissue_of, tm.tissue_of.data(), tm.tissue_of.size() * 4);
    if (bnd_dst) std::memcpy(bnd_dst, tm.bnd_dst.data(), tm.bnd_dst.size() * 8);
    if (bnd_src) std::memcpy(bnd_src, tm.bnd_src.data(), tm.bnd_src.size() * 8);
    return LQT_OK;
}
