// The single-wall RPY pair formulas of pair_math.cuh in double-float
// arithmetic (df64 mode).  Same algebra (division-free, two reciprocal square
// roots per pair); exact float constants multiply with the cheaper df x float
// product, powers of two scale exactly.
#pragma once
#include "dfloat.cuh"
#include "rmw_common.cuh"

namespace rmw {

struct dfc {
    // compile-time split of a double constant into hi + lo floats
    static constexpr df make(double d) { return {(float)d, (float)(d - (double)(float)d)}; }
};

template <int KIND>
__device__ __forceinline__ void pair_contrib_df(df dx, df dy, df dz, df Rz, df hi, df hj, df vx, df vy, df vz,
                                                df &ux, df &uy, df &uz)
{
    constexpr df ONE_THIRD = dfc::make(1.0 / 3.0);
    constexpr df TWO_THIRDS = dfc::make(2.0 / 3.0);
    constexpr df FOUR_THIRDS = dfc::make(4.0 / 3.0);
    const df dx2 = sqr(dx), dy2 = sqr(dy);
    const df rho2 = dx2 + dy2;
    const df r2 = rho2 + sqr(dz);
    const df invr = rsqrt_df(r2);
    const df r = r2 * invr;
    const df R2 = rho2 + sqr(Rz);
    const df invR = rsqrt_df(R2);
    const df invR2 = sqr(invR);
    const df ex = dx * invR, ey = dy * invR, ez = Rz * invR;
    const df ez2 = sqr(ez);
    if (KIND == RMW_UF) {
        const df invr2 = sqr(invr);
        df A, Bc;
        if (r > 2.0f) {
            A = (TWO_THIRDS * invr2 + 1.0f) * invr;
            Bc = (1.0f - scale2(invr2, 2.0f)) * invr2 * invr;
        } else {
            A = FOUR_THIRDS * (1.0f - r * 0.28125f);
            Bc = scale2(invr, 0.125f);
        }
        const df dv = dx * vx + dy * vy + dz * vz;
        const df invR3 = invR2 * invR;
        const df invR5 = invR3 * invR2;
        const df hh = hi * hj * invR2;
        const df q5 = (1.0f - ez2 * 5.0f) * invR3;  // (1 - 5 ez^2) invR^3, shared by f1, f2, f3
        const df f1 = -(((scale2(hh, 2.0f) + 1.0f) * invR) * 3.0f + scale2((1.0f - ez2 * 3.0f) * invR3, 2.0f) -
                        scale2(q5 * invR2, 2.0f)) * ONE_THIRD;
        const df f2 = -(((1.0f - hh * 6.0f) * invR) * 3.0f - q5 * 6.0f + ((1.0f - ez2 * 7.0f) * invR5) * 10.0f) *
                      ONE_THIRD;
        const df hjR2 = hj * invR2;
        const df f3 = TWO_THIRDS * (hjR2 * 3.0f - (hh * ez * invR) * 18.0f +
                                    ez * (((2.0f - ez2 * 7.0f) * invR5) * 10.0f - q5 * 6.0f));
        const df f4 = TWO_THIRDS * (hjR2 * 3.0f - (ez * invR5) * 10.0f);
        const df f5 = -FOUR_THIRDS * (((sqr(hj) + ez2) * invR3) * 3.0f + (2.0f - ez2 * 15.0f) * invR5);
        const df ev = ex * vx + ey * vy + ez * vz;
        const df ce = f2 * ev + f3 * vz;
        const df Af = A + f1;
        const df bdv = Bc * dv;
        ux = ux + (Af * vx + bdv * dx + ce * ex);
        uy = uy + (Af * vy + bdv * dy + ce * ey);
        uz = uz + (Af * vz + bdv * dz + ce * ez + f4 * ev + f5 * vz);
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        const df invr2 = sqr(invr);
        const df c = (r >= 2.0f) ? invr2 * invr : scale2(1.0f - r * 0.375f, 0.5f);
        df ax = c * (vy * dz - vz * dy);
        df ay = c * (vz * dx - vx * dz);
        df az = c * (vx * dy - vy * dx);
        const df invR3 = invR2 * invR;
        const df invR4 = sqr(invR2);
        const df h = (KIND == RMW_UT) ? hi : hj;
        const df hR3 = h * invR3;
        const df ezR4 = ez * invR4;
        const df f1 = invR2;
        const df f2 = scale2((hR3 * ez) * 6.0f + (1.0f - ez2 * 10.0f) * invR4, 2.0f);
        const df f3 = scale2(hR3 * 3.0f - ezR4 * 5.0f, -2.0f);
        const df f4 = scale2(hR3 - ezR4, -2.0f);
        const df g = f1 + f2 + f3 * ez;
        const df p = f1 * ez + f4;
        if (KIND == RMW_UT) {
            const df q = ey * vx - ex * vy;
            ax = ax + (f3 * ex * q + p * vy + f1 * ey * vz);
            ay = ay + (f3 * ey * q - p * vx - f1 * ex * vz);
            az = az - g * q;
        } else {
            const df s2 = ex * vx + ey * vy;
            ax = ax + (f3 * ey * s2 - p * vy + g * ey * vz);
            ay = ay + (p * vx - f3 * ex * s2 - g * ex * vz);
            az = az + f1 * (ex * vy - ey * vx);
        }
        ux = ux + ax;
        uy = uy + ay;
        uz = uz + az;
    } else {  // RMW_WT
        const df invr2 = sqr(invr);
        const df invr3 = invr2 * invr;
        df A, Bc;
        if (r >= 2.0f) {
            A = invr3 * -0.5f;
            Bc = (invr2 * invr3) * 1.5f;
        } else {
            A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
            Bc = invr * 0.28125f - r * 0.046875f;
        }
        const df dv = dx * vx + dy * vy + dz * vz;
        const df invR3 = invR2 * invR;
        const df f1 = scale2((1.0f - ez2 * 6.0f) * invR3, 0.5f);
        const df f2 = invR3 * -1.5f;
        const df f3 = (invR3 * ez) * 3.0f;
        const df f4 = invR3 * 3.0f;
        const df ev = ex * vx + ey * vy + ez * vz;
        const df tv = f4 * (ex * vy - ey * vx);
        const df Af = A + f1;
        const df fe = f2 * ev;
        const df bdv = Bc * dv;
        ux = ux + (Af * vx + bdv * dx + fe * ex - tv * ey);
        uy = uy + (Af * vy + bdv * dy + fe * ey + tv * ex);
        uz = uz + (Af * vz + bdv * dz + fe * ez + f3 * ev);
    }
}

}  // namespace rmw
