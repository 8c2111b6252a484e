// Pair formulas of the single-wall RPY mobility blocks (shared by the
// all-pairs product kernels and the dense per-body mobility of the
// preconditioner).
#pragma once
#include "rmw_common.cuh"

namespace rmw {

// pair math.  (dx,dy,dz) = (r_i - r_j)/a; Rz = (z_i + z_j)/a; hi = z_i/a; hj = z_j/a.
template <typename T> __device__ __forceinline__ T rsq(T x);
template <> __device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(x); }

template <int KIND, typename T>
__device__ __forceinline__ void pair_contrib(T dx, T dy, T dz, T Rz, T hi, T hj, T vx, T vy, T vz, T &ux, T &uy,
                                             T &uz)
{
    const T r2 = dx * dx + dy * dy + dz * dz;
    const T invr = rsq<T>(r2);
    const T r = r2 * invr;
    const T R2 = dx * dx + dy * dy + Rz * Rz;
    const T invR = rsq<T>(R2);
    const T invR2 = invR * invR;
    const T ex = dx * invR, ey = dy * invR, ez = Rz * invR;
    const T ez2 = ez * ez;
    if (KIND == RMW_UF) {
        const T invr2 = invr * invr;
        T A, Bc;
        if (r > T(2)) {
            A = (T(1) + T(2.0 / 3.0) * invr2) * invr;
            Bc = (T(1) - T(2) * invr2) * invr2 * invr;
        } else {
            A = T(4.0 / 3.0) * (T(1) - T(0.28125) * r);
            Bc = T(0.125) * invr;
        }
        const T dv = dx * vx + dy * vy + dz * vz;
        const T invR3 = invR2 * invR;
        const T invR5 = invR3 * invR2;
        const T hh = hi * hj * invR2;
        const T f1 = -(T(3) * (T(1) + T(2) * hh) * invR + T(2) * (T(1) - T(3) * ez2) * invR3 -
                       T(2) * (T(1) - T(5) * ez2) * invR5) * T(1.0 / 3.0);
        const T f2 = -(T(3) * (T(1) - T(6) * hh) * invR - T(6) * (T(1) - T(5) * ez2) * invR3 +
                       T(10) * (T(1) - T(7) * ez2) * invR5) * T(1.0 / 3.0);
        const T f3 = T(2.0 / 3.0) * (T(3) * hj * invR2 - T(18) * hh * ez * invR +
                                     ez * (T(10) * (T(2) - T(7) * ez2) * invR5 - T(6) * (T(1) - T(5) * ez2) * invR3));
        const T f4 = T(2.0 / 3.0) * (T(3) * hj * invR2 - T(10) * ez * invR5);
        const T f5 = T(-4.0 / 3.0) * (T(3) * (hj * hj + ez2) * invR3 + (T(2) - T(15) * ez2) * invR5);
        const T ev = ex * vx + ey * vy + ez * vz;
        const T ce = f2 * ev + f3 * vz;
        const T Af = A + f1;
        ux += Af * vx + Bc * dv * dx + ce * ex;
        uy += Af * vy + Bc * dv * dy + ce * ey;
        uz += Af * vz + Bc * dv * dz + ce * ez + f4 * ev + f5 * vz;
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        const T c = (r >= T(2)) ? invr * invr * invr : T(0.5) * (T(1) - T(0.375) * r);
        // RPY part: c (v x d)
        T ax = c * (vy * dz - vz * dy);
        T ay = c * (vz * dx - vx * dz);
        T az = c * (vx * dy - vy * dx);
        const T invR3 = invR2 * invR;
        const T invR4 = invR2 * invR2;
        const T h = (KIND == RMW_UT) ? hi : hj;  // UT evaluates the wall term with i and j swapped
        const T f1 = invR2;
        const T f2 = T(2) * (T(6) * h * invR3 * ez + (T(1) - T(10) * ez2) * invR4);
        const T f3 = T(-2) * (T(3) * h * invR3 - T(5) * ez * invR4);
        const T f4 = T(-2) * (h * invR3 - ez * invR4);
        const T g = f1 + f2 + f3 * ez;
        const T p = f1 * ez + f4;
        if (KIND == RMW_UT) {
            const T q = ey * vx - ex * vy;
            ax += f3 * ex * q + p * vy + f1 * ey * vz;
            ay += f3 * ey * q - p * vx - f1 * ex * vz;
            az -= g * q;
        } else {
            const T s2 = ex * vx + ey * vy;
            ax += f3 * ey * s2 - p * vy + g * ey * vz;
            ay += -f3 * ex * s2 + p * vx - g * ex * vz;
            az += f1 * (ex * vy - ey * vx);
        }
        ux += ax;
        uy += ay;
        uz += az;
    } else {  // RMW_WT
        const T invr2 = invr * invr;
        const T invr3 = invr2 * invr;
        T A, Bc;
        if (r >= T(2)) {
            A = T(-0.5) * invr3;
            Bc = T(1.5) * invr2 * invr3;
        } else {
            A = T(1) - T(0.84375) * r + T(0.078125) * r * r2;
            Bc = T(0.28125) * invr - T(0.046875) * r;
        }
        const T dv = dx * vx + dy * vy + dz * vz;
        const T invR3 = invR2 * invR;
        const T f1 = T(0.5) * (T(1) - T(6) * ez2) * invR3;
        const T f2 = T(-1.5) * invR3;
        const T f3 = T(3) * invR3 * ez;
        const T f4 = T(3) * invR3;
        const T ev = ex * vx + ey * vy + ez * vz;
        const T tv = f4 * (ex * vy - ey * vx);
        const T Af = A + f1;
        const T fe = f2 * ev;
        ux += Af * vx + Bc * dv * dx + fe * ex - tv * ey;
        uy += Af * vy + Bc * dv * dy + fe * ey + tv * ex;
        uz += Af * vz + Bc * dv * dz + fe * ez + f3 * ev;
    }
}

// Minimum-image projection of mobility/mobility_numba.py (int() truncates toward zero).
template <typename T> __device__ __forceinline__ T project(T d, T L)
{
    T s = (T)((d > T(0)) - (d < T(0)));
    return d - (T)(long long)(d / L + T(0.5) * s) * L;
}


}  // namespace rmw
