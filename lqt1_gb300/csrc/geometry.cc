// geometry.cc -- host preprocessing of 2D/3D tissue grids and the seeded
// synthetic geometries.
//
// Tissue numbering follows GPU3D.cu:1307-1333 (x-major, z fastest).  The
// mirror-boundary map follows GPU3D.cu:1487-1604 (3D) and new_11.cu:1535-1640
// (2D): every empty voxel with a tissue neighbour estimates an outward normal
// from the weighted occupancy of its neighbours and takes the V of the tissue
// neighbour nearest to that direction.  The sums use the reference's term
// order because last-bit ties in the nearest-voxel search depend on it.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/lqt.h"
#include "geometry.h"
#include "mirror_tables.h"

namespace lqt {

namespace {

inline int64_t gi(int64_t ny, int64_t nz, int64_t x, int64_t y, int64_t z) { return (x * ny + y) * nz + z; }

// Occupancy terms of the normal components (mirror_tables.h).
const int8_t kIc3[18][3] = LQT_MIRROR_IC3;
const int8_t kIr3[18][3] = LQT_MIRROR_IR3;
const int8_t kIl3[18][3] = LQT_MIRROR_IL3;
const int8_t kIl2[6][3] = LQT_MIRROR_IL2;
const int8_t kIr2[6][3] = LQT_MIRROR_IR2;
const int kSlot2X[9] = LQT_MIRROR_SLOT2X;
const int kSlot2Y[9] = LQT_MIRROR_SLOT2Y;

double occ_sum(const int8_t (*t)[3], int n, const int *gg)
{
    static const double r2 = std::sqrt(2.0), r3 = std::sqrt(3.0);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
        const int g = gg[t[i][0]];
        const double term = t[i][1] == 1 ? (double)g : (t[i][1] == 2 ? g / r2 : g / r3);
        acc = t[i][2] > 0 ? acc + term : acc - term;
    }
    return acc;
}

}  // namespace

int64_t build_tissue_map(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types, TissueMap &out)
{
    const int64_t total = (int64_t)nx * ny * nz;
    out.tissue_of.assign(total, -1);
    out.cells.clear();
    for (int64_t i = 0; i < total; ++i)
        if (types[i] != LQT_EMPTY) {
            out.tissue_of[i] = (int32_t)out.cells.size();
            out.cells.push_back(i);
        }
    const bool is2d = nz == 1;
    auto tissue = [&](int64_t x, int64_t y, int64_t z) {
        return x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz && types[gi(ny, nz, x, y, z)] != LQT_EMPTY;
    };
    std::vector<std::vector<std::pair<int64_t, int64_t>>> per_x(nx);
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t x = 0; x < nx; ++x) {
        auto &vec = per_x[x];
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t z = 0; z < nz; ++z) {
                if (types[gi(ny, nz, x, y, z)] != LQT_EMPTY) continue;
                int gg[27] = {0};
                int nb = 0;
                if (is2d) {
                    for (int k = 1; k <= 8; ++k) {
                        gg[k] = tissue(x + kSlot2X[k], y + kSlot2Y[k], 0);
                        nb += gg[k];
                    }
                } else {
                    int k = 0;
                    for (int ox = -1; ox <= 1; ++ox)
                        for (int oy = -1; oy <= 1; ++oy)
                            for (int oz = -1; oz <= 1; ++oz) {
                                if (!ox && !oy && !oz) continue;
                                gg[++k] = tissue(x + ox, y + oy, z + oz);
                                nb += gg[k];
                            }
                }
                if (!nb) continue;
                double il, ir, ic = 0.0, imax;
                if (is2d) {
                    il = occ_sum(kIl2, 6, gg);
                    ir = occ_sum(kIr2, 6, gg);
                    imax = std::fabs(il);
                    if (std::fabs(ir) > imax) imax = std::fabs(ir);
                } else {
                    ic = occ_sum(kIc3, 18, gg);
                    ir = occ_sum(kIr3, 18, gg);
                    il = occ_sum(kIl3, 18, gg);
                    imax = std::fabs(ic);
                    if (std::fabs(ir) > imax) imax = std::fabs(ir);
                    if (std::fabs(il) > imax) imax = std::fabs(il);
                }
                double nxv = il / imax, nyv = ir / imax, nzv = is2d ? 0.0 : ic / imax;
                if (imax - 0 < 0.0001) nxv = nyv = nzv = 0.0;
                double best = 1000;
                int bx = 0, by = 0, bz = 0;
                const int zlo = is2d ? 0 : -1, zhi = is2d ? 0 : 1;
                for (int zc = zlo; zc <= zhi; ++zc)
                    for (int yc = -1; yc <= 1; ++yc)
                        for (int xc = -1; xc <= 1; ++xc) {
                            const double dis = is2d ? std::sqrt(1.0 * (xc - nxv) * (xc - nxv) + (yc - nyv) * (yc - nyv))
                                                    : std::sqrt(1.0 * (xc - nxv) * (xc - nxv) + (yc - nyv) * (yc - nyv) +
                                                                (zc - nzv) * (zc - nzv));
                            if (tissue(x + xc, y + yc, z + zc) && dis < best) {
                                bx = xc; by = yc; bz = zc;
                                best = dis;
                            }
                        }
                vec.emplace_back(gi(ny, nz, x, y, z), gi(ny, nz, x + bx, y + by, z + bz));
            }
    }
    out.bnd_dst.clear();
    out.bnd_src.clear();
    for (auto &vec : per_x)
        for (auto &pr : vec) {
            out.bnd_dst.push_back(pr.first);
            out.bnd_src.push_back(pr.second);
        }
    return (int64_t)out.cells.size();
}

// D = d_t I + (d_f - d_t) f f^T per tissue voxel (new_11.cu:1495-1499 in 2D)
// and b_j = sum_i dD_ij/dx_i with central differences between tissue
// neighbours, one-sided beside non-tissue (new_11.cu:383-408).
void build_tensor(int32_t nx, int32_t ny, int32_t nz, double dx, const TissueMap &tm, const float *fibre,
                  double d_f, double d_t, std::vector<float> &d6, std::vector<float> &b3)
{
    const int64_t n = (int64_t)tm.cells.size();
    std::vector<double> D((size_t)n * 6);
    const double dd = d_f - d_t;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t g = tm.cells[k];
        const double f0 = fibre[3 * g], f1 = fibre[3 * g + 1], f2 = fibre[3 * g + 2];
        double *o = &D[6 * k];
        o[0] = d_t + dd * f0 * f0;
        o[1] = d_t + dd * f1 * f1;
        o[2] = d_t + dd * f2 * f2;
        o[3] = dd * f0 * f1;
        o[4] = dd * f0 * f2;
        o[5] = dd * f1 * f2;
    }
    static const int comp[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    const int64_t stride[3] = {(int64_t)ny * nz, nz, 1};
    const int32_t dims[3] = {nx, ny, nz};
    d6.resize((size_t)n * 6);
    b3.resize((size_t)n * 3);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t g = tm.cells[k];
        const int64_t c[3] = {g / ((int64_t)ny * nz), (g / nz) % ny, g % nz};
        double b[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i) {
            if (dims[i] == 1) continue;
            const int32_t tp = c[i] + 1 < dims[i] ? tm.tissue_of[g + stride[i]] : -1;
            const int32_t tmi = c[i] - 1 >= 0 ? tm.tissue_of[g - stride[i]] : -1;
            for (int j = 0; j < 3; ++j) {
                const int cc = comp[i][j];
                double der;
                if (tp >= 0 && tmi >= 0) der = (D[6 * (int64_t)tp + cc] - D[6 * (int64_t)tmi + cc]) / (2 * dx);
                else if (tp >= 0) der = (D[6 * (int64_t)tp + cc] - D[6 * k + cc]) / dx;
                else if (tmi >= 0) der = (D[6 * k + cc] - D[6 * (int64_t)tmi + cc]) / dx;
                else der = 0;
                b[j] += der;
            }
        }
        for (int j = 0; j < 6; ++j) d6[6 * k + j] = (float)D[6 * k + j];
        for (int j = 0; j < 3; ++j) b3[3 * k + j] = (float)b[j];
    }
}

}  // namespace lqt

using namespace lqt;

extern "C" {

// 2D sheet of nx*ny tissue voxels inside a grid of (nx+2)*(ny+2) with one
// empty voxel on every side: cell types in bands along x (fractions endo / M
// / epi), S1 on the first `s1_cols` tissue columns, S2 on the quadrant of
// tissue x < nx/2, y < ny/2.
int lqt_geom_sheet(int32_t nx, int32_t ny, double frac_endo, double frac_mid, int32_t s1_cols, uint8_t *types,
                   uint8_t *s1_mask, uint8_t *s2_mask)
{
    if (nx < 2 || ny < 2 || !types || frac_endo < 0 || frac_mid < 0 || frac_endo + frac_mid > 1) {
        g_err = "lqt_geom_sheet: bad arguments";
        return LQT_ERR_INVALID;
    }
    const int32_t gx = nx + 2, gy = ny + 2;
    const int32_t xe = (int32_t)std::lround(frac_endo * nx), xm = (int32_t)std::lround((frac_endo + frac_mid) * nx);
    for (int32_t X = 0; X < gx; ++X)
        for (int32_t Y = 0; Y < gy; ++Y) {
            const int64_t g = (int64_t)X * gy + Y;
            const int32_t x = X - 1, y = Y - 1;
            const bool in = x >= 0 && x < nx && y >= 0 && y < ny;
            types[g] = !in ? LQT_EMPTY : (x < xe ? LQT_ENDO : (x < xm ? LQT_MCELL : LQT_EPI));
            if (s1_mask) s1_mask[g] = in && x < s1_cols;
            if (s2_mask) s2_mask[g] = in && x < nx / 2 && y < ny / 2;
        }
    return LQT_OK;
}

// Tissue numbering and mirror map of a grid, host only (the map the
// simulation builds in lqt_sim_create).
int lqt_geom_mirror_map(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types, int32_t *tissue_of,
                        int64_t *bnd_dst, int64_t *bnd_src, int64_t *nbnd)
{
    if (nx < 1 || ny < 1 || nz < 1 || !types || !nbnd) {
        g_err = "lqt_geom_mirror_map: bad arguments";
        return LQT_ERR_INVALID;
    }
    TissueMap tm;
    build_tissue_map(nx, ny, nz, types, tm);
    *nbnd = (int64_t)tm.bnd_dst.size();
    if (tissue_of) std::memcpy(tissue_of, tm.tissue_of.data(), tm.tissue_of.size() * 4);
    if (bnd_dst) std::memcpy(bnd_dst, tm.bnd_dst.data(), tm.bnd_dst.size() * 8);
    if (bnd_src) std::memcpy(bnd_src, tm.bnd_src.data(), tm.bnd_src.size() * 8);
    return LQT_OK;
}

// Truncated prolate-ellipsoid shell (see lqt_ventricle_spec in geometry.h).
int lqt_geom_ventricle(const lqt_ventricle_spec *sp, uint8_t *types, float *fibre, uint8_t *s1_mask,
                       double *island_out)
{
    if (!sp || !types || sp->nx <= 2 || sp->ny <= 2 || sp->nz <= 2 || !(sp->dx > 0) || !(sp->wall > 0) ||
        !(sp->a_out > sp->wall) || !(sp->c_out > sp->wall)) {
        g_err = "lqt_geom_ventricle: bad arguments";
        return LQT_ERR_INVALID;
    }
    const int32_t nx = sp->nx, ny = sp->ny, nz = sp->nz;
    const double dx = sp->dx;
    const double a1 = sp->a_out, c1 = sp->c_out, a0 = a1 - sp->wall, c0 = c1 - sp->wall;
    const double cx = sp->cx, cy = sp->cy, zb = sp->z_base;
    // seeded M-cell island centre: free wall, mid-wall depth, 40-70% height
    std::mt19937_64 rng(sp->seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const double th = 2.0 * M_PI * U(rng);
    const double hfrac = 0.4 + 0.3 * U(rng);
    const double em = 0.5 * (sp->endo_frac + 1.0 - sp->epi_frac);
    const double am = a0 + em * sp->wall, cm = c0 + em * sp->wall;
    const double zi = -cm * (1.0 - hfrac);              // below the base plane
    const double ri = am * std::sqrt(std::max(0.0, 1.0 - zi * zi / (cm * cm)));
    const double isl[3] = {cx + ri * std::cos(th), cy + ri * std::sin(th), zb + zi};
    if (island_out) std::memcpy(island_out, isl, sizeof(isl));
    const double apex[3] = {cx, cy, zb - c1};
    const double alpha0 = sp->alpha_endo_deg * M_PI / 180.0, alpha1 = sp->alpha_epi_deg * M_PI / 180.0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t x = 0; x < nx; ++x)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t z = 0; z < nz; ++z) {
                const int64_t g = ((int64_t)x * ny + y) * nz + z;
                const double px = x * dx - cx, py = y * dx - cy, pz = z * dx - zb;
                const double rr = px * px + py * py;
                uint8_t t = LQT_EMPTY;
                float fv[3] = {0, 0, 0};
                uint8_t stim = 0;
                if (pz <= 0.0 && rr / (a1 * a1) + pz * pz / (c1 * c1) <= 1.0 &&
                    rr / (a0 * a0) + pz * pz / (c0 * c0) >= 1.0) {
                    // transmural depth e in [0, 1]: the shell surface through the
                    // point has semi-axes (a0 + e w, c0 + e w)
                    double lo = 0.0, hi = 1.0;
                    for (int it = 0; it < 40; ++it) {
                        const double e = 0.5 * (lo + hi);
                        const double a = a0 + e * sp->wall, c = c0 + e * sp->wall;
                        if (rr / (a * a) + pz * pz / (c * c) > 1.0) lo = e;
                        else hi = e;
                    }
                    const double e = 0.5 * (lo + hi);
                    const double dxi = x * dx - isl[0], dyi = y * dx - isl[1], dzi = z * dx - isl[2];
                    const bool in_island = dxi * dxi + dyi * dyi + dzi * dzi < sp->island_radius * sp->island_radius;
                    if (e < sp->endo_frac) t = LQT_ENDO;
                    else if (e >= 1.0 - sp->epi_frac) t = LQT_EPI;
                    else t = in_island ? LQT_MCELL : (e < em ? LQT_ENDO : LQT_EPI);
                    // fibre: circumferential rotated towards the meridian by alpha(e)
                    const double a = a0 + e * sp->wall, c = c0 + e * sp->wall;
                    double n[3] = {px / (a * a), py / (a * a), pz / (c * c)};
                    double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    for (double &q : n) q /= nn;
                    double ch[3];
                    const double rxy = std::sqrt(rr);
                    if (rxy > 1e-9) {
                        ch[0] = -py / rxy; ch[1] = px / rxy; ch[2] = 0.0;
                    } else {
                        ch[0] = 1.0; ch[1] = 0.0; ch[2] = 0.0;
                    }
                    // meridian direction: z axis projected on the tangent plane
                    double lh[3] = {-n[2] * n[0], -n[2] * n[1], 1.0 - n[2] * n[2]};
                    double ln = std::sqrt(lh[0] * lh[0] + lh[1] * lh[1] + lh[2] * lh[2]);
                    if (ln < 1e-9) {
                        lh[0] = 0; lh[1] = 1; lh[2] = 0; ln = 1;
                    }
                    for (double &q : lh) q /= ln;
                    const double al = alpha0 + (alpha1 - alpha0) * e;
                    for (int j = 0; j < 3; ++j) fv[j] = (float)(std::cos(al) * ch[j] + std::sin(al) * lh[j]);
                    const double sx = x * dx - apex[0], sy = y * dx - apex[1], sz = z * dx - apex[2];
                    stim = sx * sx + sy * sy + sz * sz <= sp->stim_radius * sp->stim_radius;
                }
                types[g] = t;
                if (fibre) {
                    fibre[3 * g] = fv[0];
                    fibre[3 * g + 1] = fv[1];
                    fibre[3 * g + 2] = fv[2];
                }
                if (s1_mask) s1_mask[g] = stim;
            }
    return LQT_OK;
}

}  // extern "C"
