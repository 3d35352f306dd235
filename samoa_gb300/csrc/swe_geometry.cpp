// Geometry tables of the Sierpinski cells: volume and edge lengths by depth, and
// the outward unit normals of the three edges for each of the 16 plotter-grammar
// orientations (src/SFC_data_types.f90:509-700).
#include <cmath>
#include <cstdint>
#include <vector>

#include "swe_internal.h"

namespace swe {

namespace {

// fl(x)^i rounded once to nearest-even: the value a Fortran compiler folds for
// the PARAMETER arrays sqrt(0.5)**i (src/SFC_data_types.f90:535,557,584).
// x = m * 2^(e-53) with an integer m; m^i is formed exactly in 32-bit limbs.
double power_rounded_once(double x, int i) {
    if (i == 0) return 1.0;
    int e;
    double f = std::frexp(x, &e);
    uint64_t m = (uint64_t)std::ldexp(f, 53);
    std::vector<uint32_t> v{1u};
    for (int k = 0; k < i; ++k) {
        uint64_t carry = 0;
        for (auto& limb : v) {
            // limb * m does not fit 64 bits; split m into two 32-bit halves
            uint64_t lo = (uint64_t)limb * (uint32_t)m;
            uint64_t hi = (uint64_t)limb * (uint32_t)(m >> 32);
            uint64_t s = lo + carry;
            uint64_t c1 = s < lo ? 1 : 0;
            limb = (uint32_t)s;
            carry = (s >> 32) + (c1 << 32) + hi;
        }
        while (carry) {
            v.push_back((uint32_t)carry);
            carry >>= 32;
        }
    }
    auto bit = [&](int64_t b) -> int { return (int)((v[(size_t)(b / 32)] >> (b % 32)) & 1u); };
    int64_t top = (int64_t)v.size() * 32 - 1;
    while (!bit(top)) --top;
    int64_t shift = top + 1 - 53;
    uint64_t q = 0;
    for (int64_t b = top; b >= shift; --b) q = (q << 1) | (uint64_t)bit(b);
    bool half = shift >= 1 && bit(shift - 1);
    bool rest = false;
    for (int64_t b = shift - 2; b >= 0 && !rest; --b) rest = bit(b) != 0;
    if (half && (rest || (q & 1))) ++q;
    return std::ldexp((double)q, (int)(shift + (int64_t)i * (e - 53)));
}

}  // namespace

void geometry_tables(double leg[kMaxDepth + 2], double vol[kMaxDepth + 1], double normal[17][3][2]) {
    const double s = std::sqrt(0.5);
    leg[0] = 1.0 / s;  // sqrt(0.5)**(-1): one correctly rounded division
    for (int i = 0; i <= kMaxDepth; ++i) leg[i + 1] = power_rounded_once(s, i);
    for (int i = 0; i <= kMaxDepth; ++i) vol[i] = std::ldexp(1.0, -(i + 1));

    // init_transform_data: Jacobian of a rotation by |p| * 45 degrees (reflected for
    // p < 0), scaled by 1.5 and truncated to whole numbers; normals are the
    // reference normals (-1,0), (1,1), (0,-1) times the inverse Jacobian, normalised.
    const double pi = 4.0 * std::atan(1.0);
    for (int p = -8; p <= 8; ++p) {
        if (p == 0) {
            for (int k = 0; k < 3; ++k) normal[8][k][0] = normal[8][k][1] = 0.0;
            continue;
        }
        const double a = pi / 4.0 * (double)std::abs(p);
        double j11, j21, j12, j22;  // J(row, col)
        if (p > 0) {
            j11 = std::cos(a); j21 = std::sin(a); j12 = -std::sin(a); j22 = std::cos(a);
        } else {
            j11 = -std::sin(a); j21 = std::cos(a); j12 = std::cos(a); j22 = std::sin(a);
        }
        j11 = std::trunc(1.5 * j11); j21 = std::trunc(1.5 * j21);
        j12 = std::trunc(1.5 * j12); j22 = std::trunc(1.5 * j22);
        const double det = j11 * j22 - j12 * j21;
        const double r = 1.0 / det;
        const double i11 = r * j22, i21 = r * -j21, i12 = r * -j12, i22 = r * j11;
        const double ref[3][2] = {{-1.0, 0.0}, {1.0, 1.0}, {0.0, -1.0}};
        for (int k = 0; k < 3; ++k) {
            // row vector times matrix, each component a sum started at +0
            double nx = 0.0;
            nx = nx + ref[k][0] * i11;
            nx = nx + ref[k][1] * i21;
            double ny = 0.0;
            ny = ny + ref[k][0] * i12;
            ny = ny + ref[k][1] * i22;
            double d = 0.0;
            d = d + nx * nx;
            d = d + ny * ny;
            const double inv = 1.0 / std::sqrt(d);
            normal[p + 8][k][0] = inv * nx;
            normal[p + 8][k][1] = inv * ny;
        }
    }
}

}  // namespace swe
