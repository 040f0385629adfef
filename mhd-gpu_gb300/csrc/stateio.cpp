// stateio.cpp - state files in the reference's formats (include/mhdgpu.h,
// mhdgpu_*_state / mhdgpu_write_result / mhdgpu_write_check), host side.
//
//   init / checkpoint file (Heterogeneous_MHD/C/init.c:33-66): raw native
//     float32, cells with x outermost and z innermost, 8 floats per cell
//     (rho, m_x, m_y, m_z, E, b_x, b_y, b_z).  mhdgpu_read_state reads it
//     (any box size; the reference hard-codes the size and the file name),
//     mhdgpu_write_state writes it, so a run can be checkpointed and resumed
//     in the same format the reference starts from;
//   result dump (C/mhd.c:126-160): two raw files, u (5 floats per cell) and
//     b (3 per cell), cells in the same x-outer, z-inner order;
//   check dump (C/check_value.c:22-79): eight text files, one per field,
//     "%8.6e\n" per cell, cells in storage order (x fastest).
// In memory the state is the reference layout u(5,nx,ny,nz), b(3,nx,ny,nz)
// (component fastest, then x, y, z).  Errors return MHD_ERR_ARG (bad
// arguments, a file of the wrong size) or MHD_ERR_NOMEM (I/O failure), with
// the message in mhdgpu_last_error().
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "mhdgpu.h"

namespace mhd {
void set_last_error(const char *msg);
}

namespace {

int io_fail(int st, const std::string &msg)
{
    mhd::set_last_error(msg.c_str());
    return st;
}

bool dims_ok(int nx, int ny, int nz)
{
    return nx >= 1 && ny >= 1 && nz >= 1 && (long long)nx * ny * nz <= (1LL << 31);
}

// storage index of cell (i, j, k)
inline size_t cell(int i, int j, int k, int nx, int ny) { return ((size_t)k * ny + j) * nx + i; }

}  // namespace

extern "C" {

int mhdgpu_read_state(const char *path, float *u, float *b, int nx, int ny, int nz)
{
    if (!path || !u || !b || !dims_ok(nx, ny, nz)) return io_fail(MHD_ERR_ARG, "mhdgpu_read_state: bad argument");
    FILE *f = fopen(path, "rb");
    if (!f) return io_fail(MHD_ERR_NOMEM, std::string("mhdgpu_read_state: cannot open ") + path);
    const size_t ncell = (size_t)nx * ny * nz;
    fseek(f, 0, SEEK_END);
    const long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (size != (long)(ncell * 8 * sizeof(float))) {
        fclose(f);
        return io_fail(MHD_ERR_ARG, "mhdgpu_read_state: file size is not 32 bytes x nx*ny*nz");
    }
    // one x-plane (ny*nz cells) at a time: the file runs z fastest, memory x fastest
    std::vector<float> plane((size_t)ny * nz * 8);
    for (int i = 0; i < nx; ++i) {
        if (fread(plane.data(), sizeof(float), plane.size(), f) != plane.size()) {
            fclose(f);
            return io_fail(MHD_ERR_NOMEM, "mhdgpu_read_state: short read");
        }
        size_t r = 0;
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k, r += 8) {
                const size_t c = cell(i, j, k, nx, ny);
                memcpy(u + 5 * c, &plane[r], 5 * sizeof(float));
                memcpy(b + 3 * c, &plane[r + 5], 3 * sizeof(float));
            }
    }
    fclose(f);
    return MHD_OK;
}

int mhdgpu_write_state(const char *path, const float *u, const float *b, int nx, int ny, int nz)
{
    if (!path || !u || !b || !dims_ok(nx, ny, nz)) return io_fail(MHD_ERR_ARG, "mhdgpu_write_state: bad argument");
    FILE *f = fopen(path, "wb");
    if (!f) return io_fail(MHD_ERR_NOMEM, std::string("mhdgpu_write_state: cannot open ") + path);
    std::vector<float> plane((size_t)ny * nz * 8);
    for (int i = 0; i < nx; ++i) {
        size_t r = 0;
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k, r += 8) {
                const size_t c = cell(i, j, k, nx, ny);
                memcpy(&plane[r], u + 5 * c, 5 * sizeof(float));
                memcpy(&plane[r + 5], b + 3 * c, 3 * sizeof(float));
            }
        if (fwrite(plane.data(), sizeof(float), plane.size(), f) != plane.size()) {
            fclose(f);
            return io_fail(MHD_ERR_NOMEM, "mhdgpu_write_state: short write");
        }
    }
    if (fclose(f) != 0) return io_fail(MHD_ERR_NOMEM, "mhdgpu_write_state: close failed");
    return MHD_OK;
}

int mhdgpu_write_result(const char *path_u, const char *path_b, const float *u, const float *b, int nx,
                        int ny, int nz)
{
    if (!path_u || !path_b || !u || !b || !dims_ok(nx, ny, nz))
        return io_fail(MHD_ERR_ARG, "mhdgpu_write_result: bad argument");
    FILE *fu = fopen(path_u, "wb");
    FILE *fb = fu ? fopen(path_b, "wb") : nullptr;
    if (!fu || !fb) {
        if (fu) fclose(fu);
        return io_fail(MHD_ERR_NOMEM, "mhdgpu_write_result: cannot open the output files");
    }
    std::vector<float> pu((size_t)ny * nz * 5), pb((size_t)ny * nz * 3);
    bool ok = true;
    for (int i = 0; i < nx && ok; ++i) {
        size_t r = 0;
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k, ++r) {
                const size_t c = cell(i, j, k, nx, ny);
                memcpy(&pu[5 * r], u + 5 * c, 5 * sizeof(float));
                memcpy(&pb[3 * r], b + 3 * c, 3 * sizeof(float));
            }
        ok = fwrite(pu.data(), sizeof(float), pu.size(), fu) == pu.size() &&
             fwrite(pb.data(), sizeof(float), pb.size(), fb) == pb.size();
    }
    ok = (fclose(fu) == 0) && ok;
    ok = (fclose(fb) == 0) && ok;
    return ok ? MHD_OK : io_fail(MHD_ERR_NOMEM, "mhdgpu_write_result: write failed");
}

int mhdgpu_write_check(const char *prefix, const float *u, const float *b, int nx, int ny, int nz)
{
    if (!prefix || !u || !b || !dims_ok(nx, ny, nz)) return io_fail(MHD_ERR_ARG, "mhdgpu_write_check: bad argument");
    static const char *names[8] = {"u1", "u2", "u3", "u4", "u5", "b1", "b2", "b3"};
    const size_t ncell = (size_t)nx * ny * nz;
    for (int fld = 0; fld < 8; ++fld) {
        const std::string path = std::string(prefix) + names[fld] + ".dat";
        FILE *f = fopen(path.c_str(), "w");
        if (!f) return io_fail(MHD_ERR_NOMEM, "mhdgpu_write_check: cannot open " + path);
        const float *src = fld < 5 ? u + fld : b + (fld - 5);
        const int stride = fld < 5 ? 5 : 3;
        bool ok = true;
        for (size_t c = 0; c < ncell && ok; ++c) ok = fprintf(f, "%8.6e\n", (double)src[c * stride]) > 0;
        ok = (fclose(f) == 0) && ok;
        if (!ok) return io_fail(MHD_ERR_NOMEM, "mhdgpu_write_check: write failed on " + path);
    }
    return MHD_OK;
}

}  // extern "C"
