// io.cu -- the reference's binary velocity-field file (.fvel) written from
// SoA host fields (src/app/PermeabilityRunner.cpp:109-159).
//
// Layout, little-endian: "FVEL", u8 version 1, u8 0, u16 0, u64 nx, ny, nz,
// f64 porosity, f64 viscosity, f64 driving[3], then N records of three f64
// (vx, vy, vz) in flat x-fastest order.  The field is interleaved in chunks
// so the staging buffer stays small for large grids.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/fftperm.h"
#include "internal.h"

namespace {

bool little_endian() {
    const uint16_t one = 1;
    unsigned char b[2];
    std::memcpy(b, &one, 2);
    return b[0] == 1;
}

}  // namespace

namespace fp {
bool write_fvel_header(void* file, int nx, int ny, int nz, double porosity, double viscosity,
                       const double driving[3]) {
    unsigned char head[72];
    std::memset(head, 0, sizeof(head));
    std::memcpy(head, "FVEL", 4);
    head[4] = 1;
    const uint64_t dims[3] = {(uint64_t)nx, (uint64_t)ny, (uint64_t)nz};
    std::memcpy(head + 8, dims, 24);
    std::memcpy(head + 32, &porosity, 8);
    std::memcpy(head + 40, &viscosity, 8);
    std::memcpy(head + 48, driving, 24);
    return std::fwrite(head, 1, sizeof(head), static_cast<std::FILE*>(file)) == sizeof(head);
}
}  // namespace fp

extern "C" int fp_write_fvel(const char* path, int nx, int ny, int nz, double porosity,
                             double viscosity, const double driving[3], const double* vx,
                             const double* vy, const double* vz) {
    if (!path || nx <= 0 || ny <= 0 || nz <= 0 || !driving || !vx || !vy || !vz)
        return FP_ERR_INVALID;
    if (!little_endian()) return FP_ERR_UNSUPPORTED;  // the format is little-endian
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return FP_ERR_INVALID;
    bool ok = fp::write_fvel_header(f, nx, ny, nz, porosity, viscosity, driving);
    const size_t n = (size_t)nx * ny * nz;
    const size_t chunk = 1 << 16;
    std::vector<double> rec(3 * chunk);
    for (size_t i0 = 0; ok && i0 < n; i0 += chunk) {
        const size_t m = n - i0 < chunk ? n - i0 : chunk;
        for (size_t i = 0; i < m; ++i) {
            rec[3 * i] = vx[i0 + i];
            rec[3 * i + 1] = vy[i0 + i];
            rec[3 * i + 2] = vz[i0 + i];
        }
        ok = std::fwrite(rec.data(), sizeof(double), 3 * m, f) == 3 * m;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FP_OK : FP_ERR_INVALID;
}
