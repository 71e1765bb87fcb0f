// Seeded D2Q9 geometry generators (host side): channel with non-overlapping disks, lid-driven
// cavity, random disks up to a solid fraction.  These produce the flag masks that the reference
// derives from a mesh (Lattice::insertModel, Lattice.cpp:228-260) for the 2-D workloads.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_capi.h"

namespace lbm {
lbm_status set_thread_error(lbm_status s, const std::string &msg);
}

namespace {

// SplitMix64 (Steele, Lea, Flood 2014): 64-bit state, one add and three xor-shift-multiply rounds
struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Disk {
    double x, y, r;
};

// visit the cells whose centre (x+0.5, y+0.5) lies inside the disk; x wraps when periodic_x
template <class F>
void raster_disk(const Disk &d, int nx, int ny, bool periodic_x, F &&visit) {
    const int y0 = std::max(0, (int)std::floor(d.y - d.r - 1.0));
    const int y1 = std::min(ny - 1, (int)std::ceil(d.y + d.r + 1.0));
    const int x0 = (int)std::floor(d.x - d.r - 1.0), x1 = (int)std::ceil(d.x + d.r + 1.0);
    for (int y = y0; y <= y1; ++y) {
        const double dy = (y + 0.5) - d.y;
        for (int xi = x0; xi <= x1; ++xi) {
            int x = xi;
            if (periodic_x) {
                x = ((x % nx) + nx) % nx;
            } else if (x < 0 || x >= nx) {
                continue;
            }
            const double dx = (xi + 0.5) - d.x;
            if (dx * dx + dy * dy <= d.r * d.r) visit((int64_t)y * nx + x);
        }
    }
}

}  // namespace

extern "C" {

LBM_API lbm_status lbm_gen_channel(int32_t nx, int32_t ny, int32_t ndisks, float rmin, float rmax, uint64_t seed,
                                   uint8_t *flags, float *disks_out) {
    if (nx < 1 || ny < 3 || ndisks < 0 || !flags || rmin < 0 || rmax < rmin)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_gen_channel: bad arguments");
    std::memset(flags, 0, (size_t)nx * ny);
    for (int x = 0; x < nx; ++x) {
        flags[x] = LBM_WALL;
        flags[(int64_t)(ny - 1) * nx + x] = LBM_WALL;
    }
    SplitMix64 rng(seed);
    std::vector<Disk> placed;
    const int64_t max_attempts = 1000000;
    for (int64_t a = 0; a < max_attempts && (int)placed.size() < ndisks; ++a) {
        Disk d{rng.u01() * nx, rng.u01() * ny, rmin + rng.u01() * (rmax - rmin)};
        bool ok = true;
        for (const Disk &p : placed) {
            double dx = std::fabs(d.x - p.x);
            dx = std::min(dx, nx - dx);  // x-periodic distance
            const double dy = d.y - p.y;
            if (dx * dx + dy * dy < (d.r + p.r) * (d.r + p.r)) {
                ok = false;
                break;
            }
        }
        if (ok) placed.push_back(d);
    }
    if ((int)placed.size() < ndisks)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_gen_channel: could not place " + std::to_string(ndisks) +
                                                          " non-overlapping disks");
    for (size_t i = 0; i < placed.size(); ++i) {
        raster_disk(placed[i], nx, ny, true, [&](int64_t c) { flags[c] = LBM_WALL; });
        if (disks_out) {
            disks_out[3 * i + 0] = (float)placed[i].x;
            disks_out[3 * i + 1] = (float)placed[i].y;
            disks_out[3 * i + 2] = (float)placed[i].r;
        }
    }
    return LBM_OK;
}

LBM_API lbm_status lbm_gen_cavity(int32_t nx, int32_t ny, uint8_t *flags) {
    if (nx < 3 || ny < 3 || !flags) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_gen_cavity: bad arguments");
    std::memset(flags, 0, (size_t)nx * ny);
    for (int y = 0; y < ny; ++y) {
        flags[(int64_t)y * nx] = LBM_WALL;
        flags[(int64_t)y * nx + nx - 1] = LBM_WALL;
    }
    for (int x = 0; x < nx; ++x) {
        flags[x] = LBM_WALL;
        flags[(int64_t)(ny - 1) * nx + x] = LBM_MOVING_WALL;
    }
    return LBM_OK;
}

LBM_API lbm_status lbm_gen_disks_fraction(int32_t nx, int32_t ny, float solid_fraction, float rmin, float rmax,
                                          uint64_t seed, uint8_t *flags, float *achieved) {
    if (nx < 1 || ny < 1 || !flags || solid_fraction < 0 || solid_fraction > 0.9f || rmin <= 0 || rmax < rmin)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_gen_disks_fraction: bad arguments");
    const int64_t n = (int64_t)nx * ny;
    auto count = [&]() {
        int64_t s = 0;
        for (int64_t i = 0; i < n; ++i) s += flags[i] != LBM_FLUID;
        return s;
    };
    SplitMix64 rng(seed);
    int64_t solid = count();
    const int64_t want = (int64_t)std::ceil((double)solid_fraction * n);
    for (int it = 0; it < 100000 && solid < want; ++it) {
        Disk d{rng.u01() * nx, rng.u01() * ny, rmin + rng.u01() * (rmax - rmin)};
        // only fluid cells become solid: walls and moving walls keep their kind
        raster_disk(d, nx, ny, false, [&](int64_t c) {
            if (flags[c] == LBM_FLUID) {
                flags[c] = LBM_WALL;
                ++solid;
            }
        });
    }
    if (achieved) *achieved = (float)((double)solid / (double)n);
    return LBM_OK;
}

}  // extern "C"
