// io.cc -- the drivers' output files, host side.
//
//   lqt_io_write_vtk  legacy-VTK structured points of V, in the layout that
//                     GPU3D.cu:123-163 (3D, every 3rd voxel per axis) and
//                     new_11.cu:142-180 (2D, every voxel) write;
//   lqt_io_write_dat  tab-separated "%4.10f" rows, the format of OneD.cc:402-415,
//                     SingleCell.cc:113-139 and OneD_VW.cc (Transmural1D files).
//
// Both write exactly the characters the reference's loops write, so files can
// be compared byte for byte.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_common.h"

using namespace lqt;

namespace lqt {

// Header + body of the reference's writeData(): DIMENSIONS use integer division
// by the stride while the loops visit every multiple of the stride (the two
// differ when an extent is not a multiple of the stride; the file then holds
// more points than the header declares, as the reference's does).  Values are
// printed as a C++ stream prints a double by default (printf "%g"), empty
// voxels as "-100", each followed by one space; a newline ends every x row and
// another every z plane.
int write_vtk_file(const char *path, const double *samples, int32_t nx, int32_t ny, int32_t nz, int32_t stride)
{
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(LQT_ERR_IO, std::string("lqt_io_write_vtk: cannot open ") + path);
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    const long long dx = nx / stride, dy = ny / stride, dz = nz / stride;
    std::fprintf(f, "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET STRUCTURED_POINTS\n");
    std::fprintf(f, "DIMENSIONS %lld %lld %lld\n", dx, dy, dz);
    std::fprintf(f, "SPACING 1 1 1\nORIGIN 0 0 0\nPOINT_DATA %lld\n", dx * dy * dz);
    std::fprintf(f, "SCALARS ImageFile float 1\nLOOKUP_TABLE default\n");
    int64_t i = 0;
    char num[64];
    for (int32_t z = 0; z < nz; z += stride) {
        for (int32_t y = 0; y < ny; y += stride) {
            for (int32_t x = 0; x < nx; x += stride) {
                // empty voxels arrive as -100.0, which "%g" prints as "-100"
                const int len = std::snprintf(num, sizeof(num), "%g ", samples[i++]);
                std::fwrite(num, 1, (size_t)len, f);
            }
            std::fputc('\n', f);
        }
        std::fputc('\n', f);
    }
    const bool ok = !std::ferror(f);
    if (std::fclose(f) != 0 || !ok) return fail(LQT_ERR_IO, std::string("lqt_io_write_vtk: write failed: ") + path);
    return LQT_OK;
}

int64_t vtk_samples(int32_t nx, int32_t ny, int32_t nz, int32_t stride)
{
    const int64_t cx = (nx + stride - 1) / stride, cy = (ny + stride - 1) / stride, cz = (nz + stride - 1) / stride;
    return cx * cy * cz;
}

}  // namespace lqt

extern "C" {

int lqt_io_write_vtk(const char *path, const double *samples_host, int32_t nx, int32_t ny, int32_t nz,
                     int32_t stride)
{
    if (!path || !samples_host || nx < 1 || ny < 1 || nz < 1 || stride < 1)
        return fail(LQT_ERR_INVALID, "lqt_io_write_vtk: NULL, or extents/stride < 1");
    return write_vtk_file(path, samples_host, nx, ny, nz, stride);
}

int lqt_io_write_dat(const char *path, int64_t nrows, int32_t ncols, const double *rows_host, int32_t append)
{
    if (!path || nrows < 0 || ncols < 1 || (nrows > 0 && !rows_host))
        return fail(LQT_ERR_INVALID, "lqt_io_write_dat: NULL or ncols < 1");
    FILE *f = std::fopen(path, append ? "a" : "w");
    if (!f) return fail(LQT_ERR_IO, std::string("lqt_io_write_dat: cannot open ") + path);
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    for (int64_t r = 0; r < nrows; ++r) {
        for (int32_t c = 0; c < ncols; ++c) std::fprintf(f, "%4.10f\t", rows_host[r * ncols + c]);
        std::fputc('\n', f);
    }
    const bool ok = !std::ferror(f);
    if (std::fclose(f) != 0 || !ok) return fail(LQT_ERR_IO, std::string("lqt_io_write_dat: write failed: ") + path);
    return LQT_OK;
}

}  // extern "C"
