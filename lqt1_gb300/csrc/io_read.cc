// io_read.cc -- readers for the reference drivers' input text files.
//
//   geometry: "x y z fx fy fz code" per tissue voxel (GPU3D.cu:1276-1296,
//             1424-1468) or, in 2D, "x y fx fy code" (new_11.cu:1296-1302,
//             1444-1478); every line is a tissue voxel;
//   stimulation profile: "x y z a b c onset tag" per stimulated point
//             (GPU3D.cu:1694-1712; new_11.cu:1723-1741 keeps layer z = 157).
//
// Lines are read one at a time; blank lines are skipped (the reference's
// `while (!feof) fscanf` loop processes its last line twice when the file ends
// with a newline, which the reference warns about; that repeat is not
// reproduced).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "api_common.h"

using namespace lqt;

namespace {

// Cell type of a geometry code (GPU3D.cu:655-1220, new_11.cu:700-1219):
// 7-10 and 17-20 epicardial, 4-6 and 14-16 M cells, everything else endocardial.
uint8_t code_type(int code)
{
    if ((code >= 7 && code <= 10) || (code >= 17 && code <= 20)) return LQT_EPI;
    if ((code >= 4 && code <= 6) || (code >= 14 && code <= 16)) return LQT_MCELL;
    return LQT_ENDO;
}

struct LineReader {
    FILE *f = nullptr;
    std::vector<char> buf = std::vector<char>(1 << 16);
    explicit LineReader(const char *path) : f(std::fopen(path, "r")) {}
    ~LineReader()
    {
        if (f) std::fclose(f);
    }
    // next non-blank line, or nullptr at the end
    const char *next()
    {
        while (std::fgets(buf.data(), (int)buf.size(), f)) {
            const char *p = buf.data();
            while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
            if (*p) return buf.data();
        }
        return nullptr;
    }
};

}  // namespace

extern "C" {

int lqt_io_read_geometry(const char *path, const lqt_geom_file_spec *sp, uint8_t *cell_type, uint8_t *code_out,
                         float *fibre, uint8_t *s2_mask, int64_t *ntissue)
{
    if (!path || !sp || !ntissue) return fail(LQT_ERR_INVALID, "lqt_io_read_geometry: NULL");
    const int dim = sp->dim;
    const int64_t nx = sp->nx, ny = sp->ny, nz = dim == 2 ? 1 : sp->nz;
    if ((dim != 2 && dim != 3) || nx < 1 || ny < 1 || nz < 1 || nx * ny * nz > (int64_t)INT32_MAX || sp->reserved)
        return fail(LQT_ERR_INVALID, "lqt_io_read_geometry: dim 2 or 3, extents >= 1, grid below 2^31, reserved 0");
    LineReader rd(path);
    if (!rd.f) return fail(LQT_ERR_IO, std::string("lqt_io_read_geometry: cannot open ") + path);
    const int64_t ng = nx * ny * nz;
    if (cell_type) std::memset(cell_type, LQT_EMPTY, ng);
    if (code_out) std::memset(code_out, 0, ng);
    if (fibre) std::memset(fibre, 0, ng * 3 * sizeof(float));
    if (s2_mask) std::memset(s2_mask, 0, ng);
    std::vector<uint8_t> seen((size_t)ng, 0);
    int64_t n = 0, lineno = 0;
    const int nf = dim == 3 ? 7 : 5;
    double v[7];
    while (const char *line = rd.next()) {
        ++lineno;
        // integers x, y (, z), doubles fx, fy (, fz), integer code
        const char *s = line;
        char *end = nullptr;
        bool ok = true;
        for (int i = 0; i < nf && ok; ++i) {
            const bool integer = i < dim || i == nf - 1;
            v[i] = integer ? (double)std::strtol(s, &end, 10) : std::strtod(s, &end);
            ok = end != s;
            s = end;
        }
        if (!ok) return fail(LQT_ERR_IO, "lqt_io_read_geometry: bad line " + std::to_string(lineno));
        const int64_t x = (int64_t)v[0], y = (int64_t)v[1], z = dim == 3 ? (int64_t)v[2] : 0;
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz)
            return fail(LQT_ERR_IO, "lqt_io_read_geometry: point outside the grid on line " + std::to_string(lineno));
        const double fx = v[dim], fy = v[dim + 1], fz = dim == 3 ? v[dim + 2] : 0.0;
        int code = (int)v[nf - 1];
        bool s2 = false;
        if (sp->case_edits) {
            if (dim == 3) {
                // GPU3D.cu:1437-1466
                s2 = x >= 300 && x < 687 && y >= 120 && y < 486 && z >= 420 && z < 534;
                if (code >= 4 && code <= 6) code = fy <= 4 ? 2 : 7;
                const double dist = std::sqrt(std::pow((double)(x - 597), 2.0) + std::pow((double)(y - 336), 2.0) +
                                              std::pow((double)(z - 336), 2.0));
                if (code >= 14 && code <= 16 && !(dist < 75)) code = code <= 14 ? 12 : 17;
            } else {
                // new_11.cu:1452-1478
                s2 = x >= 300 && x < 400 && y >= 200 && y < 350 && code <= 13 && code >= 11;
                if (code >= 3 && code <= 6) code = code <= 4 ? 2 : 7;
                if (code >= 13 && code <= 16 && !(x >= 550 && x < 689 && y >= 150 && y < 487))
                    code = code <= 14 ? 12 : 17;
            }
        }
        const int64_t g = (x * ny + y) * nz + z;
        if (seen[g]) return fail(LQT_ERR_IO, "lqt_io_read_geometry: duplicated point on line " + std::to_string(lineno));
        seen[g] = 1;
        if (cell_type) cell_type[g] = code_type(code);
        if (code_out) code_out[g] = (uint8_t)code;
        if (fibre) {
            fibre[g * 3 + 0] = (float)fx;
            fibre[g * 3 + 1] = (float)fy;
            fibre[g * 3 + 2] = (float)fz;
        }
        if (s2_mask) s2_mask[g] = s2 ? 1 : 0;
        ++n;
    }
    *ntissue = n;
    return LQT_OK;
}

int lqt_io_read_stimulation(const char *path, int32_t nx, int32_t ny, int32_t nz, int32_t layer,
                            const uint8_t *cell_type, uint8_t *s1_mask, float *onset, int64_t *npoints)
{
    if (!path || !cell_type || !npoints || nx < 1 || ny < 1 || nz < 1)
        return fail(LQT_ERR_INVALID, "lqt_io_read_stimulation: NULL or extents < 1");
    LineReader rd(path);
    if (!rd.f) return fail(LQT_ERR_IO, std::string("lqt_io_read_stimulation: cannot open ") + path);
    const int64_t ng = (int64_t)nx * ny * nz;
    if (s1_mask) std::memset(s1_mask, 0, ng);
    if (onset) std::memset(onset, 0, ng * sizeof(float));
    int64_t n = 0, lineno = 0;
    while (const char *line = rd.next()) {
        ++lineno;
        const char *s = line;
        char *end = nullptr;
        long xyz[3];
        double f[4];
        bool ok = true;
        for (int i = 0; i < 3 && ok; ++i) {
            xyz[i] = std::strtol(s, &end, 10);
            ok = end != s;
            s = end;
        }
        for (int i = 0; i < 4 && ok; ++i) {
            f[i] = (double)std::strtof(s, &end);    // read as float, GPU3D.cu:1705
            ok = end != s;
            s = end;
        }
        if (!ok) return fail(LQT_ERR_IO, "lqt_io_read_stimulation: bad line " + std::to_string(lineno));
        int64_t x = xyz[0], y = xyz[1], z = xyz[2];
        if (layer >= 0) {           // 2D: one layer of the profile (new_11.cu:1737)
            if (z != layer) continue;
            z = 0;
        }
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) continue;
        const int64_t g = ((int64_t)x * ny + y) * nz + z;
        if (cell_type[g] == LQT_EMPTY) continue;
        if (s1_mask) s1_mask[g] = 1;
        if (onset) onset[g] = (float)f[3];
        ++n;
    }
    *npoints = n;
    return LQT_OK;
}

}  // extern "C"
