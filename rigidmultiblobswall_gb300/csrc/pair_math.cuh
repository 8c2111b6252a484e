// Pair formulas of the single-wall RPY mobility blocks (shared by the
// all-pairs product kernels and the dense per-body mobility of the
// preconditioner).
#pragma once
#include "rmw_common.cuh"

namespace rmw {

// pair math.  (dx,dy,dz) = (r_i - r_j)/a; Rz = (z_i + z_j)/a; hi = z_i/a; hj = z_j/a.
template <typename T> __device__ __forceinline__ T rsq(T x);
template <> __device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float rsq<float>(float x) { return rsqrt_approx(x); }

// The reference builds each 3x3 block from unit vectors e = (dx, dy, Rz)/R and
// then multiplies by v.  Here the products are regrouped so that e never
// appears: with s = 1/R, W = dx vx + dy vy + Rz vz and Q = dy vx - dx vy,
//   (f2 (e.v) + f3 vz) e  = (f2 W s^2 + f3 vz s) (dx, dy, Rz)
// and the RPY term Bc (d.v) d shares dx vx + dy vy with W.  h_hat never
// appears either (h_hat e_z = h_j s, (1 - h_hat) e_z = h_i s).
template <int KIND, typename T>
__device__ __forceinline__ void pair_contrib(T dx, T dy, T dz, T Rz, T hi, T hj, T vx, T vy, T vz, T &ux, T &uy,
                                             T &uz)
{
    const T rho2 = dx * dx + dy * dy;
    const T r2 = rho2 + dz * dz;
    const T invr = rsq<T>(r2);
    const T r = r2 * invr;
    const T Rz2 = Rz * Rz;
    const T s = rsq<T>(rho2 + Rz2);
    const T s2 = s * s;
    const T s3 = s2 * s;
    const T E = Rz2 * s2;  // e_z^2
    const T Pxy = dx * vx + dy * vy;
    if (KIND == RMW_UF) {
        const T invr2 = invr * invr;
        // far branch always; the near (r <= 2) branch only when some lane of the
        // warp needs it (rare: touching blobs), so warps stay convergent
        T A = (T(1) + T(2.0 / 3.0) * invr2) * invr;
        T Bc = (T(1) - T(2) * invr2) * invr2 * invr;
        const bool near = !(r > T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = T(4.0 / 3.0) * (T(1) - T(0.28125) * r);
                Bc = T(0.125) * invr;
            }
        }
        const T dv = Pxy + dz * vz;
        const T W = Pxy + Rz * vz;
        const T s5 = s3 * s2;
        const T hh = hi * hj * s2;
        const T ez = Rz * s;
        const T q5 = (T(1) - T(5) * E) * s3;
        const T f1 = -((T(1) + T(2) * hh) * s + T(2.0 / 3.0) * ((T(1) - T(3) * E) * s3 - q5 * s2));
        const T f2 = -((T(1) - T(6) * hh) * s - T(2) * q5 + T(10.0 / 3.0) * (T(1) - T(7) * E) * s5);
        const T f3 = T(2.0 / 3.0) * (T(3) * hj * s2 - T(18) * hh * ez * s +
                                     ez * (T(10) * (T(2) - T(7) * E) * s5 - T(6) * q5));
        const T f4 = T(2.0 / 3.0) * (T(3) * hj * s2 - T(10) * ez * s5);
        const T f5 = T(-4.0 / 3.0) * (T(3) * (hj * hj + E) * s3 + (T(2) - T(15) * E) * s5);
        const T Af = A + f1;
        const T Gr = Bc * dv;
        const T Gw = (f2 * W * s + f3 * vz) * s;
        const T G = Gr + Gw;
        ux += Af * vx + G * dx;
        uy += Af * vy + G * dy;
        uz += Af * vz + Gr * dz + Gw * Rz + f4 * W * s + f5 * vz;
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        T c = invr * invr * invr;
        const bool near = !(r >= T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) c = T(0.5) * (T(1) - T(0.375) * r);
        }
        const T Q = dy * vx - dx * vy;  // (v x d)_z
        // RPY part: c (v x d)
        T ax = c * (vy * dz - vz * dy);
        T ay = c * (vz * dx - vx * dz);
        T az = c * Q;
        const T s4 = s2 * s2;
        const T ez = Rz * s;
        const T h = (KIND == RMW_UT) ? hi : hj;  // UT evaluates the wall term with i and j swapped
        const T hs3 = h * s3;
        const T ezs4 = ez * s4;
        const T f2 = T(2) * (T(6) * hs3 * ez + (T(1) - T(10) * E) * s4);
        const T f3 = T(-2) * (T(3) * hs3 - T(5) * ezs4);
        const T f4 = T(-2) * (hs3 - ezs4);
        const T p = s2 * ez + f4;  // f1 = s^2
        if (KIND == RMW_UT) {
            const T F3 = f3 * s2 * Q;
            const T F1 = s3 * vz;
            const T g = s2 + f2 + f3 * ez;
            ax += F3 * dx + p * vy + F1 * dy;
            ay += F3 * dy - p * vx - F1 * dx;
            az -= g * s * Q;
        } else {
            const T g = s2 + f2 + f3 * ez;
            const T H = f3 * s2 * Pxy + g * s * vz;
            ax += H * dy - p * vy;
            ay += p * vx - H * dx;
            az -= s3 * Q;
        }
        ux += ax;
        uy += ay;
        uz += az;
    } else {  // RMW_WT
        const T invr2 = invr * invr;
        const T invr3 = invr2 * invr;
        T A = T(-0.5) * invr3;
        T Bc = T(1.5) * invr2 * invr3;
        const bool near = !(r >= T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = T(1) - T(0.84375) * r + T(0.078125) * r * r2;
                Bc = T(0.28125) * invr - T(0.046875) * r;
            }
        }
        const T dv = Pxy + dz * vz;
        const T W = Pxy + Rz * vz;
        const T Q = dy * vx - dx * vy;
        const T s5 = s3 * s2;
        const T Af = A + T(0.5) * (T(1) - T(6) * E) * s3;
        const T Gw = T(-1.5) * s5 * W;
        const T Tq = T(3) * s5 * Q;
        const T Gr = Bc * dv;
        ux += Af * vx + (Gr + Gw) * dx + Tq * dy;
        uy += Af * vy + (Gr + Gw) * dy - Tq * dx;
        uz += Af * vz + Gr * dz - Gw * Rz;
    }
}

// Vector-independent part of one M_UF block, times 3/2 (the consumers'
// finalize kernels multiply the pair sums by 2/3 in FP64), for the FP32 pair
// kernels:  (3/2) M v = Af v + (Bc (d.v) + c2 W + c3 vz) (dx, dy, .) ...
// with W = dx vx + dy vy + Rz vz (see uf_apply).  The 3/2 turns the RPY and
// Swan-Brady constants into the small integers and halves below; the same
// coefficients as the double-float pair_uf_sym_df:
//   (3/2) A  = 3/(2r) + 1/r^3,          (3/2) Bc = (3/2 - 3/r^2) / r^3
//   (3/2) f1 = -(3/2 + 3 hh) s - [(1 - 3E) t - (1 - 5E) p]
//   (3/2) f2 = -(3/2 - 9 hh) s + 3 (1 - 5E) t - 5 (1 - 7E) p
//   c3 = (3/2) f3 s = 3 h_j t - 18 hh Rz t + Rz s^2 [10 (2 - 7E) p - 6 (1 - 5E) t]
//   c4 = (3/2) f4 s = 3 h_j t - 10 Rz s^2 p
//   (3/2) f5 = -2 [3 (h_j^2 + E) t + (2 - 15E) p]
// with t = s^3, p = s^5, E = (Rz s)^2, hh = h_i h_j s^2; for r <= 2
// (3/2) A = 2 (1 - 9r/32), (3/2) Bc = 3 / (16 r).
constexpr double kUFCoeffScale = 2.0 / 3.0;  // undoes the 3/2
template <typename T> struct UFCoeffs {
    T Af, Bc, c2, c3, c4, Af5;  // Af5 = Af + f5, the zz diagonal
};

template <typename T>
__device__ __forceinline__ UFCoeffs<T> uf_coeffs(T dx, T dy, T dz, T Rz, T hi, T hj)
{
    const T rho2 = dx * dx + dy * dy;
    const T r2 = rho2 + dz * dz;
    const T invr = rsq<T>(r2);
    const T Rz2 = Rz * Rz;
    const T s = rsq<T>(rho2 + Rz2);
    const T u = s * s;
    const T t = u * s;
    const T p = t * u;
    const T E = Rz2 * u;
    const T invr2 = invr * invr;
    const T invr3 = invr2 * invr;
    T A = T(1.5) * invr + invr3;
    T Bc = (T(1.5) - T(3) * invr2) * invr3;
    const bool near = !(r2 > T(4));  // r <= 2
    if (__any_sync(__activemask(), near)) {
        if (near) {
            const T r = r2 * invr;
            A = T(2) - T(0.5625) * r;
            Bc = T(0.1875) * invr;
        }
    }
    const T hh = hi * hj * u;
    const T q5 = (T(1) - T(5) * E) * t;
    const T Ru = Rz * u;
    const T hjt3 = T(3) * hj * t;
    const T f1 = -((T(1.5) + T(3) * hh) * s + ((T(1) - T(3) * E) * t - q5 * u));
    const T f2 = T(3) * q5 - (T(1.5) - T(9) * hh) * s - T(5) * (T(1) - T(7) * E) * p;
    const T c3 = hjt3 - T(18) * hh * Rz * t + Ru * (T(10) * (T(2) - T(7) * E) * p - T(6) * q5);
    const T c4 = hjt3 - T(10) * Ru * p;
    const T f5 = T(-2) * (T(3) * (hj * hj + E) * t + (T(2) - T(15) * E) * p);
    const T Af = A + f1;
    return {Af, Bc, f2 * u, c3, c4, Af + f5};
}

template <typename T>
__device__ __forceinline__ void uf_apply(const UFCoeffs<T> &c, T dx, T dy, T dz, T Rz, T vx, T vy, T vz, T &ux,
                                         T &uy, T &uz)
{
    const T Pxy = dx * vx + dy * vy;
    const T Gr = c.Bc * (Pxy + dz * vz);
    const T W = Pxy + Rz * vz;
    const T Gw = c.c2 * W + c.c3 * vz;
    const T G = Gr + Gw;
    ux += c.Af * vx + G * dx;
    uy += c.Af * vy + G * dy;
    uz += c.Af5 * vz + Gr * dz + Gw * Rz + c.c4 * W;
}

// The explicit 3x3 block of uf_coeffs, for products with several right-hand
// sides: nine FMAs per right-hand side instead of sixteen.  With d = (dx, dy,
// dz), e = (dx, dy, Rz) and z the wall normal,
//   M = Af I + Bc d d^T + c2 e e^T + c3 e z^T + c4 z e^T + f5 z z^T,
// so M_xy = M_yx = (Bc + c2) dx dy, M_xz = dx t3, M_zx = dx t4 with
// t3,4 = Bc dz + c2 Rz + c3,4, and M_zz = Af + f5 + Bc dz^2 + (c2 Rz + c3 + c4) Rz.
struct UFBlock {
    float xx, xy, xz, yy, yz, zx, zy, zz;  // M_yx = M_xy
};

__device__ __forceinline__ UFBlock uf_block_f(const UFCoeffs<float> &c, float dx, float dy, float dz, float Rz)
{
    const float b2 = c.Bc + c.c2;
    const float t = fmaf(c.Bc, dz, c.c2 * Rz);
    const float t3 = t + c.c3, t4 = t + c.c4;
    const float px = b2 * dx;
    UFBlock m;
    m.xx = fmaf(px, dx, c.Af);
    m.xy = px * dy;
    m.yy = fmaf(b2 * dy, dy, c.Af);
    m.xz = dx * t3;
    m.yz = dy * t3;
    m.zx = dx * t4;
    m.zy = dy * t4;
    m.zz = fmaf(fmaf(c.c2, Rz, c.c3 + c.c4), Rz, fmaf(c.Bc * dz, dz, c.Af5));
    return m;
}

// (ux, uy, uz) += M v
__device__ __forceinline__ void uf_block_apply(const UFBlock &m, float vx, float vy, float vz, float &ux, float &uy,
                                               float &uz)
{
    ux = fmaf(m.xx, vx, fmaf(m.xy, vy, fmaf(m.xz, vz, ux)));
    uy = fmaf(m.xy, vx, fmaf(m.yy, vy, fmaf(m.yz, vz, uy)));
    uz = fmaf(m.zx, vx, fmaf(m.zy, vy, fmaf(m.zz, vz, uz)));
}

// FP32: every term chained into the accumulator by an FMA (two plain
// multiplies and one subtraction per application)
template <>
__device__ __forceinline__ void uf_apply<float>(const UFCoeffs<float> &c, float dx, float dy, float dz, float Rz,
                                                float vx, float vy, float vz, float &ux, float &uy, float &uz)
{
    // with dv = d.v, G = Bc dv + Gw and Rz - dz = 2 h_j:
    // (M v)_z = Af5 vz + G dz + Gw (Rz - dz) + c4 W
    const float h2 = Rz - dz;
    const float dv = fmaf(dz, vz, fmaf(dy, vy, dx * vx));
    const float W = fmaf(h2, vz, dv);
    const float Gw = fmaf(c.c2, W, c.c3 * vz);
    const float G = fmaf(c.Bc, dv, Gw);
    ux = fmaf(c.Af, vx, fmaf(G, dx, ux));
    uy = fmaf(c.Af, vy, fmaf(G, dy, uy));
    uz = fmaf(c.Af5, vz, fmaf(G, dz, fmaf(Gw, h2, fmaf(c.c4, W, uz))));
}

// ---------------------------------------------------------------------------
// Symmetric forms of the rotation blocks in FP32 and FP64 (the double-float
// forms are pair_rot_sym_df): M_ji is the M_ij formula with d -> -d and
// h_i <-> h_j, so one pair evaluation serves both targets.  WT has no height
// dependence; UT and WF form the height-dependent coefficients for both
// heights.
template <typename T> __device__ __forceinline__ T fm(T a, T b, T c);
template <> __device__ __forceinline__ float fm<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double fm<double>(double a, double b, double c) { return fma(a, b, c); }

template <typename T> struct RotH {
    T f3s2, p, gs;  // f3 s^2, p = s^2 ez + f4, g s with g = s^2 + f2 + f3 ez
};
template <typename T>
__device__ __forceinline__ RotH<T> rot_h(T h, T s, T s2, T s3, T ez, T ezs4, T K)
{
    const T hs3 = h * s3;
    const T f2 = T(2) * fm<T>(T(6) * hs3, ez, K);
    const T f3 = T(-2) * fm<T>(T(3), hs3, T(-5) * ezs4);
    const T f4 = T(-2) * (hs3 - ezs4);
    const T p = fm<T>(s2, ez, f4);
    const T g = fm<T>(f3, ez, s2 + f2);
    return {f3 * s2, p, g * s};
}

template <typename T>
__device__ __forceinline__ void ut_apply(T c, const RotH<T> &H, T s3, T dx, T dy, T dz, T vx, T vy, T vz, T &ux,
                                         T &uy, T &uz)
{
    const T Q = fm<T>(dy, vx, -dx * vy);  // (v x d)_z
    const T X = fm<T>(vy, dz, -vz * dy), Y = fm<T>(vz, dx, -vx * dz);
    const T F3 = H.f3s2 * Q, F1 = s3 * vz;
    ux = fm<T>(c, X, fm<T>(F3, dx, fm<T>(F1, dy, fm<T>(H.p, vy, ux))));
    uy = fm<T>(c, Y, fm<T>(F3, dy, fm<T>(-F1, dx, fm<T>(-H.p, vx, uy))));
    uz = fm<T>(c - H.gs, Q, uz);
}

template <typename T>
__device__ __forceinline__ void wf_apply(T c, const RotH<T> &H, T s3, T dx, T dy, T dz, T vx, T vy, T vz, T &ux,
                                         T &uy, T &uz)
{
    const T Pxy = fm<T>(dy, vy, dx * vx);
    const T Q = fm<T>(dy, vx, -dx * vy);
    const T X = fm<T>(vy, dz, -vz * dy), Y = fm<T>(vz, dx, -vx * dz);
    const T Hh = fm<T>(H.f3s2, Pxy, H.gs * vz);
    ux = fm<T>(c, X, fm<T>(Hh, dy, fm<T>(-H.p, vy, ux)));
    uy = fm<T>(c, Y, fm<T>(H.p, vx, fm<T>(-Hh, dx, uy)));
    uz = fm<T>(c - s3, Q, uz);
}

template <typename T>
__device__ __forceinline__ void wt_apply(T Af, T Bc, T s5, T dx, T dy, T dz, T Rz, T vx, T vy, T vz, T &ux, T &uy,
                                         T &uz)
{
    const T Pxy = fm<T>(dy, vy, dx * vx);
    const T dv = fm<T>(dz, vz, Pxy);
    const T W = fm<T>(Rz, vz, Pxy);
    const T Q = fm<T>(dy, vx, -dx * vy);
    const T Gw = T(-1.5) * s5 * W;
    const T Tq = T(3) * s5 * Q;
    const T Gr = Bc * dv;
    const T G = Gr + Gw;
    ux = fm<T>(Af, vx, fm<T>(G, dx, fm<T>(Tq, dy, ux)));
    uy = fm<T>(Af, vy, fm<T>(G, dy, fm<T>(-Tq, dx, uy)));
    uz = fm<T>(Af, vz, fm<T>(Gr, dz, fm<T>(-Gw, Rz, uz)));
}

// UT, WF or WT for both orders of one pair: (ux, uy, uz) += M_ij v_j,
// (wx, wy, wz) += M_ji v_i.
template <typename T, int KIND>
__device__ __forceinline__ void pair_rot_sym(T dx, T dy, T dz, T Rz, T hi, T hj, T vx, T vy, T vz, T qx, T qy, T qz,
                                             T &ux, T &uy, T &uz, T &wx, T &wy, T &wz)
{
    const T rho2 = fm<T>(dx, dx, dy * dy);
    const T r2 = fm<T>(dz, dz, rho2);
    const T invr = rsq<T>(r2);
    const T Rz2 = Rz * Rz;
    const T s = rsq<T>(rho2 + Rz2);
    const T s2 = s * s, s3 = s2 * s, E = Rz2 * s2;
    const bool near = !(r2 >= T(4));  // r < 2
    if (KIND == RMW_WT) {
        const T invr2 = invr * invr, invr3 = invr2 * invr;
        T A = T(-0.5) * invr3;
        T Bc = T(1.5) * invr2 * invr3;
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const T r = r2 * invr;
                A = T(1) - T(0.84375) * r + T(0.078125) * r * r2;
                Bc = T(0.28125) * invr - T(0.046875) * r;
            }
        }
        const T s5 = s3 * s2;
        const T Af = fm<T>(T(0.5) * s3, fm<T>(T(-6), E, T(1)), A);
        wt_apply<T>(Af, Bc, s5, dx, dy, dz, Rz, vx, vy, vz, ux, uy, uz);
        wt_apply<T>(Af, Bc, s5, -dx, -dy, -dz, Rz, qx, qy, qz, wx, wy, wz);
    } else {
        T c = invr * invr * invr;
        if (__any_sync(__activemask(), near)) {
            if (near) c = T(0.5) * (T(1) - T(0.375) * (r2 * invr));
        }
        const T s4 = s2 * s2, ez = Rz * s, ezs4 = ez * s4;
        const T K = fm<T>(T(-10), E, T(1)) * s4;
        const RotH<T> Hi = rot_h<T>(hi, s, s2, s3, ez, ezs4, K);
        const RotH<T> Hj = rot_h<T>(hj, s, s2, s3, ez, ezs4, K);
        if (KIND == RMW_UT) {
            ut_apply<T>(c, Hi, s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
            ut_apply<T>(c, Hj, s3, -dx, -dy, -dz, qx, qy, qz, wx, wy, wz);
        } else {
            wf_apply<T>(c, Hj, s3, dx, dy, dz, vx, vy, vz, ux, uy, uz);
            wf_apply<T>(c, Hi, s3, -dx, -dy, -dz, qx, qy, qz, wx, wy, wz);
        }
    }
}

// Free-space blocks for both orders of one pair (the symmetric no-wall
// kernels): M_ji = M_ij(-d), so UF and WT (even in d) apply the same block to
// the other vector and UT / WF (odd in d) its negative.  (ux, uy, uz) +=
// M_ij v, (wx, wy, wz) += M_ji q.
template <typename T, int KIND>
__device__ __forceinline__ void pair_rpy_sym(T dx, T dy, T dz, T vx, T vy, T vz, T qx, T qy, T qz, T &ux, T &uy,
                                             T &uz, T &wx, T &wy, T &wz)
{
    const T r2 = fm<T>(dx, dx, fm<T>(dy, dy, dz * dz));
    const T invr = rsq<T>(r2);
    if (KIND == RMW_UT || KIND == RMW_WF) {
        T c = invr * invr * invr;
        const bool near = !(r2 >= T(4));  // r < 2
        if (__any_sync(__activemask(), near)) {
            if (near) c = T(0.5) * (T(1) - T(0.375) * (r2 * invr));
        }
        ux = fm<T>(c, fm<T>(vy, dz, -vz * dy), ux);
        uy = fm<T>(c, fm<T>(vz, dx, -vx * dz), uy);
        uz = fm<T>(c, fm<T>(dy, vx, -dx * vy), uz);
        wx = fm<T>(-c, fm<T>(qy, dz, -qz * dy), wx);
        wy = fm<T>(-c, fm<T>(qz, dx, -qx * dz), wy);
        wz = fm<T>(-c, fm<T>(dy, qx, -dx * qy), wz);
        return;
    }
    const T invr2 = invr * invr;
    T A, Bc;
    if (KIND == RMW_UF) {
        A = (T(1) + T(2.0 / 3.0) * invr2) * invr;
        Bc = (T(1) - T(2) * invr2) * invr2 * invr;
        const bool near = !(r2 > T(4));  // r <= 2
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const T r = r2 * invr;
                A = T(4.0 / 3.0) * (T(1) - T(0.28125) * r);
                Bc = T(0.125) * invr;
            }
        }
    } else {  // RMW_WT
        const T invr3 = invr2 * invr;
        A = T(-0.5) * invr3;
        Bc = T(1.5) * invr2 * invr3;
        const bool near = !(r2 >= T(4));
        if (__any_sync(__activemask(), near)) {
            if (near) {
                const T r = r2 * invr;
                A = T(1) - T(0.84375) * r + T(0.078125) * r * r2;
                Bc = T(0.28125) * invr - T(0.046875) * r;
            }
        }
    }
    const T G = Bc * fm<T>(dx, vx, fm<T>(dy, vy, dz * vz));
    const T Gq = Bc * fm<T>(dx, qx, fm<T>(dy, qy, dz * qz));
    ux = fm<T>(A, vx, fm<T>(G, dx, ux));
    uy = fm<T>(A, vy, fm<T>(G, dy, uy));
    uz = fm<T>(A, vz, fm<T>(G, dz, uz));
    wx = fm<T>(A, qx, fm<T>(Gq, dx, wx));
    wy = fm<T>(A, qy, fm<T>(Gq, dy, wy));
    wz = fm<T>(A, qz, fm<T>(Gq, dz, wz));
}

// Free-space RPY blocks (no wall): the RPY parts of pair_contrib, for the
// no-wall products (mobility/mobility_numba.py:13-1190).  (dx, dy, dz) =
// (r_i - r_j)/a.  Accumulates M_ij v into (ux, uy, uz), unscaled.
template <int KIND, typename T>
__device__ __forceinline__ void pair_rpy(T dx, T dy, T dz, T vx, T vy, T vz, T &ux, T &uy, T &uz)
{
    const T r2 = dx * dx + dy * dy + dz * dz;
    const T invr = rsq<T>(r2);
    const T r = r2 * invr;
    const T dv = dx * vx + dy * vy + dz * vz;
    if (KIND == RMW_UF) {
        const T invr2 = invr * invr;
        T A = (T(1) + T(2.0 / 3.0) * invr2) * invr;
        T Bc = (T(1) - T(2) * invr2) * invr2 * invr;
        const bool near = !(r > T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = T(4.0 / 3.0) * (T(1) - T(0.28125) * r);
                Bc = T(0.125) * invr;
            }
        }
        const T G = Bc * dv;
        ux += A * vx + G * dx;
        uy += A * vy + G * dy;
        uz += A * vz + G * dz;
    } else if (KIND == RMW_UT || KIND == RMW_WF) {
        T c = invr * invr * invr;
        const bool near = !(r >= T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) c = T(0.5) * (T(1) - T(0.375) * r);
        }
        ux += c * (vy * dz - vz * dy);
        uy += c * (vz * dx - vx * dz);
        uz += c * (dy * vx - dx * vy);
    } else {  // RMW_WT
        const T invr2 = invr * invr;
        const T invr3 = invr2 * invr;
        T A = T(-0.5) * invr3;
        T Bc = T(1.5) * invr2 * invr3;
        const bool near = !(r >= T(2));
        if (__any_sync(__activemask(), near)) {
            if (near) {
                A = T(1) - T(0.84375) * r + T(0.078125) * r * r2;
                Bc = T(0.28125) * invr - T(0.046875) * r;
            }
        }
        const T G = Bc * dv;
        ux += A * vx + G * dx;
        uy += A * vy + G * dy;
        uz += A * vz + G * dz;
    }
}

// Minimum-image projection of mobility/mobility_numba.py (int() truncates toward zero).
template <typename T> __device__ __forceinline__ T project(T d, T L)
{
    T s = (T)((d > T(0)) - (d < T(0)));
    return d - (T)(long long)(d / L + T(0.5) * s) * L;
}


}  // namespace rmw
