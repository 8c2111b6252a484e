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

// Writes the pair's contribution M_ij v_j (unscaled) to (ux, uy, uz).
template <int KIND>
__device__ __forceinline__ void pair_contrib_df(df dx, df dy, df dz, df Rz, df hi, df hj, df vx, df vy, df vz,
                                                df &ux, df &uy, df &uz)
{
    constexpr df TWO_THIRDS = dfc::make(2.0 / 3.0);
    constexpr df FOUR_THIRDS = dfc::make(4.0 / 3.0);
    constexpr df TEN_THIRDS = dfc::make(10.0 / 3.0);
    const df rho2 = mad(dx, dx, sqr(dy));
    const df r2 = mad(dz, dz, rho2);
    const df invr = rsqrt_df(r2);
    const df r = r2 * invr;
    const df Rz2 = sqr(Rz);
    const df s = rsqrt_df(rho2 + Rz2);
    const df s2 = sqr(s);
    const df s3 = s2 * s;
    const df E = Rz2 * s2;  // e_z^2
    const df Pxy = mad2(dx, vx, dy, vy);
    if (KIND == RMW_UF) {
        const df invr2 = sqr(invr);
        df A = mad(TWO_THIRDS, invr2, df_from(1.0f)) * invr;
        df Bc = (1.0f - scale2(invr2, 2.0f)) * invr2 * invr;
        const bool near = !(r > 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = FOUR_THIRDS * (1.0f - r * 0.28125f);
                Bc = scale2(invr, 0.125f);
            }
        }
        const df dv = mad(dz, vz, Pxy);
        const df W = mad(Rz, vz, Pxy);
        const df s5 = s3 * s2;
        const df hh = hi * hj * s2;
        const df ez = Rz * s;
        const df q5 = (1.0f - E * 5.0f) * s3;
        const df f1 = -mad(scale2(hh, 2.0f) + 1.0f, s, TWO_THIRDS * ((1.0f - E * 3.0f) * s3 - q5 * s2));
        const df f2 = -(mad((1.0f - hh * 6.0f), s, -scale2(q5, 2.0f)) + TEN_THIRDS * ((1.0f - E * 7.0f) * s5));
        const df f3 = TWO_THIRDS * (hj * s2 * 3.0f - (hh * ez * s) * 18.0f +
                                    ez * (((2.0f - E * 7.0f) * s5) * 10.0f - q5 * 6.0f));
        const df f4 = TWO_THIRDS * (hj * s2 * 3.0f - (ez * s5) * 10.0f);
        const df f5 = -FOUR_THIRDS * mad((sqr(hj) + E) * 3.0f, s3, (2.0f - E * 15.0f) * s5);
        const df Af = A + f1;
        const df Gr = Bc * dv;
        const df Gw = mad(f2 * W, s, f3 * vz) * s;
        const df G = Gr + Gw;
        ux = mad2(Af, vx, G, dx);
        uy = mad2(Af, vy, G, dy);
        uz = mad2(Af, vz, Gr, dz) + mad2(Gw, Rz, f4 * W, s) + f5 * vz;
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        df c = sqr(invr) * invr;
        const bool near = !(r >= 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) c = scale2(1.0f - r * 0.375f, 0.5f);
        }
        const df Q = mad2(dy, vx, -dx, vy);  // (v x d)_z
        df ax = c * mad2(vy, dz, -vz, dy);
        df ay = c * mad2(vz, dx, -vx, dz);
        df az = c * Q;
        const df s4 = sqr(s2);
        const df ez = Rz * s;
        const df h = (KIND == RMW_UT) ? hi : hj;
        const df hs3 = h * s3;
        const df ezs4 = ez * s4;
        const df f2 = scale2(mad(hs3 * 6.0f, ez, (1.0f - E * 10.0f) * s4), 2.0f);
        const df f3 = scale2(hs3 * 3.0f - ezs4 * 5.0f, -2.0f);
        const df f4 = scale2(hs3 - ezs4, -2.0f);
        const df p = mad(s2, ez, f4);
        const df g = mad(f3, ez, s2 + f2);
        if (KIND == RMW_UT) {
            const df F3 = f3 * s2 * Q;
            const df F1 = s3 * vz;
            ax = ax + mad2(F3, dx, F1, dy) + p * vy;
            ay = ay + mad2(F3, dy, -F1, dx) - p * vx;
            az = az - g * s * Q;
        } else {
            const df H = mad2(f3 * s2, Pxy, g * s, vz);
            ax = ax + mad2(H, dy, -p, vy);
            ay = ay + mad2(p, vx, -H, dx);
            az = az - s3 * Q;
        }
        ux = ax;
        uy = ay;
        uz = az;
    } else {  // RMW_WT
        const df invr2 = sqr(invr);
        const df invr3 = invr2 * invr;
        df A = invr3 * -0.5f;
        df Bc = (invr2 * invr3) * 1.5f;
        const bool near = !(r >= 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
                Bc = invr * 0.28125f - r * 0.046875f;
            }
        }
        const df dv = mad(dz, vz, Pxy);
        const df W = mad(Rz, vz, Pxy);
        const df Q = mad2(dy, vx, -dx, vy);
        const df s5 = s3 * s2;
        const df Af = A + scale2((1.0f - E * 6.0f) * s3, 0.5f);
        const df Gw = (s5 * W) * -1.5f;
        const df Tq = (s5 * Q) * 3.0f;
        const df Gr = Bc * dv;
        const df G = Gr + Gw;
        ux = mad2(Af, vx, G, dx) + Tq * dy;
        uy = mad2(Af, vy, G, dy) - Tq * dx;
        uz = mad2(Af, vz, Gr, dz) - Gw * Rz;
    }
}

// Free-space RPY block (no wall) in double-float: writes M_ij v (unscaled) to
// (ux, uy, uz); the double-float form of pair_rpy (pair_math.cuh).
template <int KIND>
__device__ __forceinline__ void pair_rpy_df(df dx, df dy, df dz, df vx, df vy, df vz, df &ux, df &uy, df &uz)
{
    constexpr df TWO_THIRDS = dfc::make(2.0 / 3.0);
    constexpr df FOUR_THIRDS = dfc::make(4.0 / 3.0);
    const df r2 = mad(dz, dz, mad(dx, dx, sqr(dy)));
    const df invr = rsqrt_df(r2);
    const df r = r2 * invr;
    const df dv = mad(dz, vz, mad2(dx, vx, dy, vy));
    if (KIND == RMW_UF) {
        const df invr2 = sqr(invr);
        df A = mad(TWO_THIRDS, invr2, df_from(1.0f)) * invr;
        df Bc = (1.0f - scale2(invr2, 2.0f)) * invr2 * invr;
        const bool near = !(r > 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = FOUR_THIRDS * (1.0f - r * 0.28125f);
                Bc = scale2(invr, 0.125f);
            }
        }
        const df G = Bc * dv;
        ux = mad2(A, vx, G, dx);
        uy = mad2(A, vy, G, dy);
        uz = mad2(A, vz, G, dz);
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        df c = sqr(invr) * invr;
        const bool near = !(r >= 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) c = scale2(1.0f - r * 0.375f, 0.5f);
        }
        ux = c * mad2(vy, dz, -vz, dy);
        uy = c * mad2(vz, dx, -vx, dz);
        uz = c * mad2(dy, vx, -dx, vy);
    } else {
        const df invr2 = sqr(invr);
        const df invr3 = invr2 * invr;
        df A = invr3 * -0.5f;
        df Bc = (invr2 * invr3) * 1.5f;
        const bool near = !(r >= 2.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
                Bc = invr * 0.28125f - r * 0.046875f;
            }
        }
        const df G = Bc * dv;
        ux = mad2(A, vx, G, dx);
        uy = mad2(A, vy, G, dy);
        uz = mad2(A, vz, G, dz);
    }
}

// UF for both orders of one pair, accumulated: (ux, uy, uz) += (3/2) M_ij v_j
// for target i and (wx, wy, wz) += (3/2) M_ji v_i = (3/2) M_ij^T v_i for
// target j (the wall mobility is symmetric).  In block form
//   M_ij = Af I + Bc d d^T + c2 e e^T + c3 e z^T + c4 z e^T + f5 z z^T
// with e = (dx, dy, Rz), z the wall normal, c2 = f2 s^2, c3 = f3 s and
// c4 = f4 s, so the transpose only swaps c3 and c4: the coefficients are
// formed once for both.  With Gw = c2 (e.v) + c3 vz and G = Bc (d.v) + Gw,
//   M v = Af v + G (dx, dy, dz) + (0, 0, Af5 vz + Gw (Rz - dz) + c4 (e.v)),
// Af5 = Af + f5 and Rz - dz = 2 h_j.  Every coefficient is formed times 3/2,
// which turns the RPY and Swan-Brady constants (2/3, 4/3, 10/3 ...) into
// exact floats; the finalize kernel multiplies the pair sums by 2/3 in FP64.
// In powers of s (t = s^3, p = s^5, E = (Rz s)^2, hh = h_i h_j s^2):
//   (3/2) A  = 3/(2r) + 1/r^3,          (3/2) Bc = (3/2 - 3/r^2) / r^3
//   (3/2) f1 = -(3/2 + 3 hh) s - [(1 - 3E) t - (1 - 5E) p]
//   (3/2) f2 = -(3/2 - 9 hh) s + 3 (1 - 5E) t - 5 (1 - 7E) p
//   (3/2) c3 = 3 h_j t - 18 hh Rz t + Rz s^2 [10 (2 - 7E) p - 6 (1 - 5E) t]
//   (3/2) c4 = 3 h_j t - 10 Rz s^2 p
//   (3/2) f5 = -2 [3 (h_j^2 + E) t + (2 - 15E) p]
// and for r <= 2: (3/2) A = 2 (1 - 9r/32), (3/2) Bc = 3 / (16 r).
// The accumulators stay unnormalised (acc_dot2 / acc_dot4, as acc_add).
struct UFCoeffsDF {
    df Af, Af5, Bc, c2, c3, c4, hj2;  // times 3/2; hj2 = Rz - dz = 2 h_j
};

__device__ __forceinline__ UFCoeffsDF uf_coeffs_df(df dx, df dy, df dz, df Rz, df hi, df hj)
{
    // mul_u / sqr_u / mad_u / add_u / sub_u: values that feed a sum directly (see dfloat.cuh)
    const df rho2 = mad_u(dx, dx, sqr_u(dy));
    const df r2 = mad(dz, dz, rho2);
    const df invr = rsqrt_df(r2);
    const df Rz2 = sqr(Rz);
    const df s = rsqrt_df(rho2 + Rz2);
    const df u = sqr(s);
    const df t = u * s;
    const df p = t * u;
    const df E = Rz2 * u;
    const df invr2 = sqr(invr);
    const df invr3 = invr2 * invr;
    df A = mad_u(invr, 1.5f, invr3);
    df Bc = (1.5f - mul_u(invr2, 3.0f)) * invr3;
    const bool near = !(r2 > 4.0f);  // r <= 2
    if (__any_sync(__activemask(), near)) {
        if (near) {
            const df r = r2 * invr;
            A = scale2(1.0f - r * 0.28125f, 2.0f);
            Bc = invr * 0.1875f;
        }
    }
    const df hh = (hi * hj) * u;
    const df q5 = (1.0f - mul_u(E, 5.0f)) * t;
    const df E7 = mul_u(E, 7.0f);
    const df f1 = -mad_u(mad(hh, 3.0f, df_from(1.5f)), s, sub_u(mul_u(1.0f - mul_u(E, 3.0f), t), mul_u(q5, u)));
    const df f2 = mad(q5, 3.0f, -mad_u(mad(hh, -9.0f, df_from(1.5f)), s, mul_u((1.0f - E7) * p, 5.0f)));
    const df f5 = scale2(mad_u((sqr_u(hj) + E) * 3.0f, t, mul_u(2.0f - mul_u(E, 15.0f), p)), -2.0f);
    const df Ru = Rz * u;
    const df hjt3 = mul_u(hj * t, 3.0f);
    UFCoeffsDF C;
    C.c4 = hjt3 - mul_u(Ru * p, 10.0f);
    C.c3 = sub_u(hjt3, mul_u(hh * (Rz * t), 18.0f)) + mul_u(Ru, mul_u((2.0f - E7) * p, 10.0f) - mul_u(q5, 6.0f));
    C.Af = A + f1;
    C.Af5 = C.Af + f5;  // the zz diagonal
    C.Bc = Bc;
    C.c2 = f2 * u;
    C.hj2 = scale2(hj, 2.0f);
    return C;
}

// (ux, uy, uz) += (3/2) M v with the coefficients of uf_coeffs_df; (c3, c4)
// exchanged gives the transposed block
__device__ __forceinline__ void uf_apply_df(const UFCoeffsDF &C, df c3, df c4, df dx, df dy, df dz, df vx, df vy,
                                            df vz, df &ux, df &uy, df &uz)
{
    const df dv = dot3(dx, vx, dy, vy, dz, vz);
    const df W = mad(C.hj2, vz, dv);  // e.v
    const df Gw = mad2(C.c2, W, c3, vz);
    const df G = mad(C.Bc, dv, Gw);
    acc_dot2(ux, C.Af, vx, G, dx);
    acc_dot2(uy, C.Af, vy, G, dy);
    acc_dot4(uz, C.Af5, vz, G, dz, Gw, C.hj2, c4, W);
}

__device__ __forceinline__ void pair_uf_sym_df(df dx, df dy, df dz, df Rz, df hi, df hj, df vx, df vy, df vz,
                                               df qx, df qy, df qz, df &ux, df &uy, df &uz, df &wx, df &wy,
                                               df &wz)
{
    const UFCoeffsDF C = uf_coeffs_df(dx, dy, dz, Rz, hi, hj);
    uf_apply_df(C, C.c3, C.c4, dx, dy, dz, vx, vy, vz, ux, uy, uz);  // M_ij v_j
    uf_apply_df(C, C.c4, C.c3, dx, dy, dz, qx, qy, qz, wx, wy, wz);  // M_ij^T v_i
}

// ---------------------------------------------------------------------------
// Symmetric forms of the rotation blocks.  With d = r_i - r_j, M_ji is the
// same formula as M_ij with d -> -d and h_i <-> h_j (the grand mobility is
// symmetric, M_ji = M_ij^T): the WT coefficients do not involve the heights,
// so its reverse block only flips d; the UT and WF coefficients depend on one
// height (UT: the target's, WF: the source's), so both height sets are formed
// and the reverse block uses the other one.  Shared per pair: the distances,
// both reciprocal square roots and the powers of s = 1/|R|.

// The height-dependent coefficients of UT / WF for height h (unnormalised
// where only a sum consumes them).
struct RotHDF {
    df f3s2, p, gs;  // f3 s^2, p = s^2 ez + f4, g s with g = f3 ez + s^2 + f2
};
__device__ __forceinline__ RotHDF rot_h_df(df h, df s, df s2, df s3, df ez, df ezs4, df K)
{
    const df hs3 = h * s3;
    const df f2 = scale2(mad_u(hs3 * 6.0f, ez, K), 2.0f);
    const df f3 = scale2(mul_u(hs3, 3.0f) - mul_u(ezs4, 5.0f), -2.0f);
    const df f4 = scale2(sub_u(hs3, ezs4), -2.0f);
    const df p = mad(s2, ez, f4);
    const df g = mad(f3, ez, s2 + f2);
    return {f3 * s2, p, g * s};
}

// (ux, uy, uz) += M_UT v for the pair (d, coefficient set H)
__device__ __forceinline__ void ut_apply_df(df c, const RotHDF &H, df s3, df dx, df dy, df dz, df vx, df vy, df vz,
                                            df &ux, df &uy, df &uz)
{
    const df Q = mad2(dy, vx, -dx, vy);  // (v x d)_z
    const df X = mad2(vy, dz, -vz, dy), Y = mad2(vz, dx, -vx, dz);
    const df F3 = H.f3s2 * Q, F1 = s3 * vz;
    acc_dot4(ux, c, X, F3, dx, F1, dy, H.p, vy);
    acc_dot4(uy, c, Y, F3, dy, F1, -dx, H.p, -vx);
    acc_dot2(uz, c, Q, H.gs, -Q);
}

// (ux, uy, uz) += M_WF v for the pair (d, coefficient set H)
__device__ __forceinline__ void wf_apply_df(df c, const RotHDF &H, df s3, df dx, df dy, df dz, df vx, df vy, df vz,
                                            df &ux, df &uy, df &uz)
{
    const df Pxy = mad2(dx, vx, dy, vy);
    const df Q = mad2(dy, vx, -dx, vy);
    const df X = mad2(vy, dz, -vz, dy), Y = mad2(vz, dx, -vx, dz);
    const df Hh = mad2(H.f3s2, Pxy, H.gs, vz);
    acc_dot3(ux, c, X, Hh, dy, H.p, -vy);
    acc_dot3(uy, c, Y, H.p, vx, Hh, -dx);
    acc_dot2(uz, c, Q, s3, -Q);
}

// (ux, uy, uz) += M_WT v for the pair (d; Af = A + (1 - 6E) s^3 / 2, Bc, s^5)
__device__ __forceinline__ void wt_apply_df(df Af, df Bc, df s5, df dx, df dy, df dz, df Rz, df vx, df vy, df vz,
                                            df &ux, df &uy, df &uz)
{
    const df Pxy = mad2(dx, vx, dy, vy);
    const df dv = mad(dz, vz, Pxy);
    const df W = mad(Rz, vz, Pxy);
    const df Q = mad2(dy, vx, -dx, vy);
    const df Gw = (s5 * W) * -1.5f;
    const df Tq = (s5 * Q) * 3.0f;
    const df Gr = Bc * dv;
    const df G = Gr + Gw;
    acc_dot3(ux, Af, vx, G, dx, Tq, dy);
    acc_dot3(uy, Af, vy, G, dy, Tq, -dx);
    acc_dot3(uz, Af, vz, Gr, dz, Gw, -Rz);
}

// UT, WF or WT for both orders of one pair: (ux, uy, uz) += M_ij v_j for
// target i, (wx, wy, wz) += M_ji v_i for target j.
template <int KIND>
__device__ __forceinline__ void pair_rot_sym_df(df dx, df dy, df dz, df Rz, df hi, df hj, df vx, df vy, df vz,
                                                df qx, df qy, df qz, df &ux, df &uy, df &uz, df &wx, df &wy,
                                                df &wz)
{
    const df rho2 = mad_u(dx, dx, sqr_u(dy));
    const df r2 = mad(dz, dz, rho2);
    const df invr = rsqrt_df(r2);
    const df Rz2 = sqr(Rz);
    const df s = rsqrt_df(rho2 + Rz2);
    const df s2 = sqr(s);
    const df s3 = s2 * s;
    const df E = Rz2 * s2;
    const bool near = !(r2 >= 4.0f);  // r < 2
    if (KIND == RMW_WT) {
        const df invr2 = sqr(invr);
        const df invr3 = invr2 * invr;
        df A = invr3 * -0.5f;
        df Bc = (invr2 * invr3) * 1.5f;
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const df r = r2 * invr;
                A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
                Bc = invr * 0.28125f - r * 0.046875f;
            }
        }
        const df s5 = s3 * s2;
        const df Af = A + scale2((1.0f - E * 6.0f) * s3, 0.5f);
        wt_apply_df(Af, Bc, s5, dx, dy, dz, Rz, vx, vy, vz, ux, uy, uz);
        wt_apply_df(Af, Bc, s5, -dx, -dy, -dz, Rz, qx, qy, qz, wx, wy, wz);
    } else {
        df c = sqr(invr) * invr;
        if (__any_sync(__activemask(), near)) {
            if (near) c = scale2(1.0f - (r2 * invr) * 0.375f, 0.5f);
        }
        const df s4 = sqr(s2);
        const df ez = Rz * s;
        const df ezs4 = ez * s4;
        const df K = mul_u(1.0f - mul_u(E, 10.0f), s4);
        const RotHDF Hi = rot_h_df(hi, s, s2, s3, ez, ezs4, K);
        const RotHDF Hj = rot_h_df(hj, s, s2, s3, ez, ezs4, K);
        if (KIND == RMW_UT) {
            ut_apply_df(c, Hi, s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
            ut_apply_df(c, Hj, s3, -dx, -dy, -dz, qx, qy, qz, wx, wy, wz);
        } else {
            wf_apply_df(c, Hj, s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
            wf_apply_df(c, Hi, s3, -dx, -dy, -dz, qx, qy, qz, wx, wy, wz);
        }
    }
}

// ---------------------------------------------------------------------------
// One-sided accumulating forms for the standard (all ordered pairs) kernels:
// (ux, uy, uz) += M_ij v_j, for UF times 3/2 (the finalize applies 2/3) with
// the coefficients and applies of the symmetric forms.
template <int KIND>
__device__ __forceinline__ void pair_acc_df(df dx, df dy, df dz, df Rz, df hi, df hj, df vx, df vy, df vz, df &ux,
                                            df &uy, df &uz)
{
    if (KIND == RMW_UF) {
        const UFCoeffsDF C = uf_coeffs_df(dx, dy, dz, Rz, hi, hj);
        uf_apply_df(C, C.c3, C.c4, dx, dy, dz, vx, vy, vz, ux, uy, uz);
        return;
    }
    const df rho2 = mad_u(dx, dx, sqr_u(dy));
    const df r2 = mad(dz, dz, rho2);
    const df invr = rsqrt_df(r2);
    const df Rz2 = sqr(Rz);
    const df s = rsqrt_df(rho2 + Rz2);
    const df s2 = sqr(s);
    const df s3 = s2 * s;
    const df E = Rz2 * s2;
    const bool near = !(r2 >= 4.0f);  // r < 2
    if (KIND == RMW_WT) {
        const df invr2 = sqr(invr);
        const df invr3 = invr2 * invr;
        df A = invr3 * -0.5f;
        df Bc = (invr2 * invr3) * 1.5f;
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const df r = r2 * invr;
                A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
                Bc = invr * 0.28125f - r * 0.046875f;
            }
        }
        const df Af = A + scale2((1.0f - E * 6.0f) * s3, 0.5f);
        wt_apply_df(Af, Bc, s3 * s2, dx, dy, dz, Rz, vx, vy, vz, ux, uy, uz);
    } else {
        df c = sqr(invr) * invr;
        if (__any_sync(__activemask(), near)) {
            if (near) c = scale2(1.0f - (r2 * invr) * 0.375f, 0.5f);
        }
        const df s4 = sqr(s2);
        const df ez = Rz * s;
        const df ezs4 = ez * s4;
        const df K = mul_u(1.0f - mul_u(E, 10.0f), s4);
        if (KIND == RMW_UT) ut_apply_df(c, rot_h_df(hi, s, s2, s3, ez, ezs4, K), s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
        else wf_apply_df(c, rot_h_df(hj, s, s2, s3, ez, ezs4, K), s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
    }
}

// Double-float form of pair_rpy_sym (free space, both orders of one pair).
template <int KIND>
__device__ __forceinline__ void pair_rpy_sym_df(df dx, df dy, df dz, df vx, df vy, df vz, df qx, df qy, df qz,
                                                df &ux, df &uy, df &uz, df &wx, df &wy, df &wz)
{
    constexpr df TWO_THIRDS = dfc::make(2.0 / 3.0);
    constexpr df FOUR_THIRDS = dfc::make(4.0 / 3.0);
    const df r2 = mad(dz, dz, mad_u(dx, dx, sqr_u(dy)));
    const df invr = rsqrt_df(r2);
    if (KIND == RMW_UT || KIND == RMW_WF) {
        df c = sqr(invr) * invr;
        const bool near = !(r2 >= 4.0f);  // r < 2
        if (__any_sync(__activemask(), near)) {
            if (near) c = scale2(1.0f - (r2 * invr) * 0.375f, 0.5f);
        }
        // c (v x d) for target i, -c (q x d) for target j
        acc_add(ux, c * mad2(vy, dz, -vz, dy));
        acc_add(uy, c * mad2(vz, dx, -vx, dz));
        acc_add(uz, c * mad2(dy, vx, -dx, vy));
        acc_add(wx, -(c * mad2(qy, dz, -qz, dy)));
        acc_add(wy, -(c * mad2(qz, dx, -qx, dz)));
        acc_add(wz, -(c * mad2(dy, qx, -dx, qy)));
        return;
    }
    const df invr2 = sqr(invr);
    df A, Bc;
    if (KIND == RMW_UF) {
        A = mad(TWO_THIRDS, invr2, df_from(1.0f)) * invr;
        Bc = (1.0f - scale2(invr2, 2.0f)) * invr2 * invr;
        const bool near = !(r2 > 4.0f);  // r <= 2
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const df r = r2 * invr;
                A = FOUR_THIRDS * (1.0f - r * 0.28125f);
                Bc = scale2(invr, 0.125f);
            }
        }
    } else {  // RMW_WT
        const df invr3 = invr2 * invr;
        A = invr3 * -0.5f;
        Bc = (invr2 * invr3) * 1.5f;
        const bool near = !(r2 >= 4.0f);
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const df r = r2 * invr;
                A = (1.0f - r * 0.84375f) + (r * r2) * 0.078125f;
                Bc = invr * 0.28125f - r * 0.046875f;
            }
        }
    }
    const df G = Bc * dot3(dx, vx, dy, vy, dz, vz);
    const df Gq = Bc * dot3(dx, qx, dy, qy, dz, qz);
    acc_dot2(ux, A, vx, G, dx);
    acc_dot2(uy, A, vy, G, dy);
    acc_dot2(uz, A, vz, G, dz);
    acc_dot2(wx, A, qx, Gq, dx);
    acc_dot2(wy, A, qy, Gq, dy);
    acc_dot2(wz, A, qz, Gq, dz);
}

}  // namespace rmw
