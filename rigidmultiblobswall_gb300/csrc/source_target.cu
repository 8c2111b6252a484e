// Translational products from forces on source blobs to velocities of target
// blobs with per-blob radii (the unequal-sphere Rotne-Prager-Yamakawa block),
// in three geometries, and the single-radius free-surface product:
//
// * free space     mobility/mobility_numba.py:1480-1572 (wall = 0), wrapper
//                  mobility/mobility.py:593-616
// * single wall    the same plus the image system of :1573-1653, with the
//                  heights shifted to max(z, radius) and forces / velocities
//                  damped by z / radius below the radius (mobility.py:87-119,
//                  551-590, pycuda twin mobility.py:494-530)
// * free surface   mobility_numba.py:1941-2093 (mobility.py:1409-1429): the
//                  pair block at the mirror image (dx, dy, z_t + z_s) times
//                  diag(1, 1, -1) added
// * free surface, one radius   mobility_numba.py:1770-1938 (mobility.py:533-548,
//                  1390-1406): the previous with every radius a and the blobs
//                  their own sources (a blob on itself takes the 4/3 self block)
//
// Pair block (a = target radius, b = source radius, r = target - source):
//   r > a+b            C1 = (1 + (a^2+b^2)/(3r^2))/r, C2 = (1 - (a^2+b^2)/r^2)/r^3
//   |b-a| < r <= a+b   C1 = (4/3)/(ab) [(a+b)/2 - ((b-a)^2 + 3r^2)^2/(32 r^3)],
//                      C2 = ((b-a)^2 - r^2)^2/(8 r^5 ab)
//   else               C1 = (4/3)/max(a,b), C2 = 0
// M = C1 I + C2 r r^T, u_t = 1/(8 pi eta) sum_s M f_s.  The wall image system
// is applied in a regrouped form, M -= W diag(1,1,-1) with
// W = al I + be e e^T + ga r e^T + de e r^T + ep r r^T at the image vector r
// (coefficients in st_wall below), algebraically identical to the
// reference's term-by-term expression and division-free after one 1/sqrt.
//
// Layout: one thread per target, sources staged through shared memory in
// tiles, the source range split over gridDim.y when there are few targets;
// a finalize kernel sums the chunks in fixed order (deterministic), scales by
// 1/(8 pi eta) and damps.  Precision modes as the other products: FP64, df64
// (double-float pair arithmetic) and mixed (FP32 pairs on double-float
// coordinate differences, compensated sums).
#include <algorithm>

#include "dfloat.cuh"
#include "pair_math.cuh"
#include "rmw_common.cuh"

namespace rmw {

namespace {

constexpr int kStThreads = 128;
constexpr int kStTile = 128;
constexpr int kGeomNoWall = 0, kGeomWall = 1, kGeomFree = 2;

// ---- arithmetic traits: one pair routine for double, float and double-float
template <typename T> struct Num;
template <> struct Num<double> {
    static __device__ __forceinline__ double k(double v) { return v; }
    static __device__ __forceinline__ double rsq(double x) { return 1.0 / sqrt(x); }
    static __device__ __forceinline__ bool gt(double a, double b) { return a > b; }
    static __device__ __forceinline__ double tabs(double a) { return fabs(a); }
    static __device__ __forceinline__ double tmin(double a, double b) { return a < b ? a : b; }
    static __device__ __forceinline__ double zero() { return 0.0; }
};
template <> struct Num<float> {
    static __device__ __forceinline__ float k(double v) { return (float)v; }
    static __device__ __forceinline__ float rsq(float x) { return rsqrt_approx(x); }
    static __device__ __forceinline__ bool gt(float a, float b) { return a > b; }
    static __device__ __forceinline__ float tabs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float tmin(float a, float b) { return a < b ? a : b; }
    static __device__ __forceinline__ float zero() { return 0.f; }
};
template <> struct Num<df> {
    static __device__ __forceinline__ df k(double v) { return df_of_double(v); }
    static __device__ __forceinline__ df rsq(df x) { return rsqrt_df(x); }
    static __device__ __forceinline__ bool gt(df a, df b) { return (a - b) > 0.0f; }
    static __device__ __forceinline__ df tabs(df a) { return a.hi < 0.0f ? -a : a; }
    static __device__ __forceinline__ df tmin(df a, df b) { return gt(a, b) ? b : a; }
    static __device__ __forceinline__ df zero() { return df_from(0.0f); }
};

// Radii-dependent constants of one target or source blob.
template <typename T> struct Rad {
    T r, r2, inv;  // radius, radius^2, 1/radius
};

// (C1, C2) of the pair block at squared distance r2 (ir = 1/sqrt(r2); r2 = 0
// gives NaN in r, which no comparison accepts: the inner branch).
template <typename T>
__device__ __forceinline__ void st_coeffs(T r2, T ir, const Rad<T> &A, const Rad<T> &B, T &C1, T &C2)
{
    using N = Num<T>;
    const T r = r2 * ir;
    const T ir2 = ir * ir, ir3 = ir2 * ir;
    if (N::gt(r, A.r + B.r)) {
        const T S = A.r2 + B.r2;
        C1 = (N::k(1.0) + S * ir2 * N::k(1.0 / 3.0)) * ir;
        C2 = (N::k(1.0) - S * ir2) * ir3;
    } else {
        const T d = B.r - A.r;
        const T inv_ab = A.inv * B.inv;
        if (N::gt(r, N::tabs(d))) {
            const T d2 = d * d;
            const T q = d2 + N::k(3.0) * r2;
            const T p = d2 - r2;
            C1 = N::k(4.0 / 3.0) * inv_ab * (N::k(0.5) * (A.r + B.r) - q * q * ir3 * N::k(1.0 / 32.0));
            C2 = p * p * (ir3 * ir2) * inv_ab * N::k(0.125);
        } else {
            C1 = N::k(4.0 / 3.0) * N::tmin(A.inv, B.inv);
            C2 = N::zero();
        }
    }
}

// u += (C1 I + C2 r r^T) g
template <typename T>
__device__ __forceinline__ void st_block(T rx, T ry, T rz, const Rad<T> &A, const Rad<T> &B, T gx, T gy, T gz,
                                         T &ux, T &uy, T &uz)
{
    const T r2 = rx * rx + ry * ry + rz * rz;
    T C1, C2;
    st_coeffs(r2, Num<T>::rsq(r2), A, B, C1, C2);
    const T rg = C2 * (rx * gx + ry * gy + rz * gz);
    ux = ux + C1 * gx + rg * rx;
    uy = uy + C1 * gy + rg * ry;
    uz = uz + C1 * gz + rg * rz;
}

// u -= W g: the single-wall image system at image vector (rx, ry, R),
// R = h + s, h / s the target / source heights.
template <typename T>
__device__ __forceinline__ void st_wall(T rx, T ry, T R, T h, T s, const Rad<T> &A, const Rad<T> &B, T gx, T gy,
                                        T gz, T &ux, T &uy, T &uz)
{
    using N = Num<T>;
    const T r2 = rx * rx + ry * ry + R * R;
    const T ir = N::rsq(r2);
    const T ir2 = ir * ir, ir3 = ir2 * ir, ir5 = ir3 * ir2, ir7 = ir5 * ir2, ir9 = ir7 * ir2;
    const T S = A.r2 + B.r2;
    const T ca = N::k(2.0 / 3.0) * A.r2, cb = N::k(2.0 / 3.0) * B.r2;
    const T cab = ca * B.r2;
    const T q = ca * s + cb * h;
    const T hs = h * s;
    const T RR = R * R;
    const T al = (N::k(1.0) + S * ir2 * N::k(1.0 / 3.0)) * ir + N::k(2.0) * hs * ir3 - N::k(3.0) * R * q * ir5 +
                 cab * (N::k(5.0) * RR * ir7 - ir5);
    const T be = N::zero() - (N::k(2.0) * ir + (ca + cb) * ir3 + N::k(2.0) * cab * ir5);
    const T c10 = N::k(10.0) * cab * R * ir7;
    const T ga = N::k(3.0) * (ca * R - q) * ir5 + c10 - N::k(2.0) * h * ir3;
    const T de = N::k(3.0) * (cb * R - q) * ir5 + c10 - N::k(2.0) * s * ir3;
    const T ep = (N::k(1.0) - S * ir2) * ir3 - N::k(6.0) * hs * ir5 + N::k(15.0) * R * q * ir7 +
                 cab * (N::k(5.0) * ir7 - N::k(35.0) * RR * ir9);
    const T rg = rx * gx + ry * gy + R * gz;
    const T t1 = be * gz + de * rg;
    const T t2 = ga * gz + ep * rg;
    ux = ux - (al * gx + t2 * rx);
    uy = uy - (al * gy + t2 * ry);
    uz = uz - (al * gz + t1 + t2 * R);
}

// One (target, source) interaction at separation (dx, dy, dz); R = h + s.
template <int GEOM, typename T>
__device__ __forceinline__ void st_pair(T dx, T dy, T dz, T R, T h, T s, const Rad<T> &A, const Rad<T> &B, T fx,
                                        T fy, T fz, T &ux, T &uy, T &uz)
{
    st_block(dx, dy, dz, A, B, fx, fy, fz, ux, uy, uz);
    if (GEOM == kGeomWall) st_wall(dx, dy, R, h, s, A, B, fx, fy, Num<T>::zero() - fz, ux, uy, uz);
    if (GEOM == kGeomFree) st_block(dx, dy, R, A, B, fx, fy, Num<T>::zero() - fz, ux, uy, uz);
}

struct StPer {
    double Lx, Ly, Lz;
};

// every periodic image of a separation: minimum image, then the neighbouring boxes
template <typename T, typename F>
__device__ __forceinline__ void st_images(T dx, T dy, T dz, T Lx, T Ly, T Lz, F &&f)
{
    if (Lx > T(0)) dx = project(dx, Lx);
    if (Ly > T(0)) dy = project(dy, Ly);
    if (Lz > T(0)) dz = project(dz, Lz);
    const int px = Lx > T(0), py = Ly > T(0), pz = Lz > T(0);
    for (int bx = -px; bx <= px; ++bx)
        for (int by = -py; by <= py; ++by)
            for (int bz = -pz; bz <= pz; ++bz) f(dx + bx * Lx, dy + by * Ly, dz + bz * Lz);
}

// ---- packed blob records (shifted heights; damped source forces) --------
struct __align__(16) StRecD {
    double x, y, z, rad;
    double fx, fy, fz, inv;
};
struct __align__(16) StRecF {
    float4 hi;  // x, y, z, radius
    float4 lo;  // coordinate remainders, 1/radius
    float4 f;   // force
};
struct __align__(16) StRecDF {
    float4 hi, lo;    // x, y, z, radius as double-float
    float4 fhi, flo;  // force, 1/radius as double-float
};

struct StBlob {
    double x, y, z, rad, inv, fx, fy, fz;
};

// position (height shifted for the wall), radius and damped force of blob i
__device__ __forceinline__ StBlob st_read(const double *__restrict__ r, const double *__restrict__ f,
                                          const double *__restrict__ rad, double rad_uniform, int i, int geom)
{
    StBlob b;
    b.x = r[3 * i];
    b.y = r[3 * i + 1];
    b.z = r[3 * i + 2];
    b.rad = rad ? rad[i] : rad_uniform;
    b.inv = 1.0 / b.rad;
    b.fx = f ? f[3 * i] : 0.0;
    b.fy = f ? f[3 * i + 1] : 0.0;
    b.fz = f ? f[3 * i + 2] : 0.0;
    if (geom == kGeomWall) {
        if (b.z < b.rad) {
            const double damp = b.z / b.rad;
            b.fx *= damp;
            b.fy *= damp;
            b.fz *= damp;
        }
        b.z = (b.z > b.rad) ? b.z : b.rad;
    }
    return b;
}

__global__ void st_pack_fp64_kernel(const double *__restrict__ r, const double *__restrict__ f,
                                    const double *__restrict__ rad, double rad_uniform, int n, int geom,
                                    StRecD *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StBlob b = st_read(r, f, rad, rad_uniform, i, geom);
    out[i] = StRecD{b.x, b.y, b.z, b.rad, b.fx, b.fy, b.fz, b.inv};
}

__global__ void st_pack_mixed_kernel(const double *__restrict__ r, const double *__restrict__ f,
                                     const double *__restrict__ rad, double rad_uniform, int n, int geom,
                                     StRecF *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StBlob b = st_read(r, f, rad, rad_uniform, i, geom);
    const float xh = (float)b.x, yh = (float)b.y, zh = (float)b.z;
    StRecF s;
    s.hi = make_float4(xh, yh, zh, (float)b.rad);
    s.lo = make_float4((float)(b.x - (double)xh), (float)(b.y - (double)yh), (float)(b.z - (double)zh),
                       (float)b.inv);
    s.f = make_float4((float)b.fx, (float)b.fy, (float)b.fz, 0.f);
    out[i] = s;
}

__global__ void st_pack_df_kernel(const double *__restrict__ r, const double *__restrict__ f,
                                  const double *__restrict__ rad, double rad_uniform, int n, int geom,
                                  StRecDF *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StBlob b = st_read(r, f, rad, rad_uniform, i, geom);
    const df x = df_of_double(b.x), y = df_of_double(b.y), z = df_of_double(b.z), ra = df_of_double(b.rad);
    const df fx = df_of_double(b.fx), fy = df_of_double(b.fy), fz = df_of_double(b.fz), iv = df_of_double(b.inv);
    StRecDF s;
    s.hi = make_float4(x.hi, y.hi, z.hi, ra.hi);
    s.lo = make_float4(x.lo, y.lo, z.lo, ra.lo);
    s.fhi = make_float4(fx.hi, fy.hi, fz.hi, iv.hi);
    s.flo = make_float4(fx.lo, fy.lo, fz.lo, iv.lo);
    out[i] = s;
}

// ---- pair kernels: thread = target, blockIdx.y = source chunk -------------
template <int GEOM, bool PER>
__global__ void __launch_bounds__(kStThreads) st_pair_fp64_kernel(const StRecD *__restrict__ trg, int nt,
                                                                   const StRecD *__restrict__ src, int ns, int chunk,
                                                                   StPer P, double *__restrict__ partial)
{
    __shared__ StRecD tile[kStTile];
    const int i = blockIdx.x * kStThreads + threadIdx.x;
    const bool valid = i < nt;
    const int j0 = blockIdx.y * chunk, j1 = min(ns, j0 + chunk);
    StRecD me = valid ? trg[i] : StRecD{0.0, 0.0, 1.0e6, 1.0, 0.0, 0.0, 0.0, 1.0};
    const Rad<double> A{me.rad, me.rad * me.rad, me.inv};
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kStTile) {
        const int cnt = min(kStTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kStThreads) tile[k] = src[t0 + k];
        __syncthreads();
        for (int k = 0; k < cnt; ++k) {
            const StRecD s = tile[k];
            const Rad<double> B{s.rad, s.rad * s.rad, s.inv};
            const double R = me.z + s.z;
            if (!PER) {
                st_pair<GEOM, double>(me.x - s.x, me.y - s.y, me.z - s.z, R, me.z, s.z, A, B, s.fx, s.fy, s.fz, ux,
                                      uy, uz);
            } else {
                st_images(me.x - s.x, me.y - s.y, me.z - s.z, P.Lx, P.Ly, P.Lz,
                          [&](double ex, double ey, double ez) {
                              st_pair<GEOM, double>(ex, ey, ez, R, me.z, s.z, A, B, s.fx, s.fy, s.fz, ux, uy, uz);
                          });
            }
        }
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * nt + 3 * (size_t)i;
        o[0] = ux;
        o[1] = uy;
        o[2] = uz;
    }
}

template <int GEOM, bool PER>
__global__ void __launch_bounds__(kStThreads) st_pair_mixed_kernel(const StRecF *__restrict__ trg, int nt,
                                                                    const StRecF *__restrict__ src, int ns, int chunk,
                                                                    StPer P, double *__restrict__ partial)
{
    __shared__ StRecF tile[kStTile];
    const int i = blockIdx.x * kStThreads + threadIdx.x;
    const bool valid = i < nt;
    const int j0 = blockIdx.y * chunk, j1 = min(ns, j0 + chunk);
    float4 mh = make_float4(0.f, 0.f, 1.0e6f, 1.f), ml = make_float4(0.f, 0.f, 0.f, 1.f);
    if (valid) {
        mh = trg[i].hi;
        ml = trg[i].lo;
    }
    const Rad<float> A{mh.w, mh.w * mh.w, ml.w};
    const float Lx = (float)P.Lx, Ly = (float)P.Ly, Lz = (float)P.Lz;
    float sx = 0.f, sy = 0.f, sz = 0.f, ex_ = 0.f, ey_ = 0.f, ez_ = 0.f;
    for (int t0 = j0; t0 < j1; t0 += kStTile) {
        const int cnt = min(kStTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kStThreads) tile[k] = src[t0 + k];
        __syncthreads();
        float ux = 0.f, uy = 0.f, uz = 0.f;
        for (int k = 0; k < cnt; ++k) {
            const float4 sh = tile[k].hi, sl = tile[k].lo, sf = tile[k].f;
            const Rad<float> B{sh.w, sh.w * sh.w, sl.w};
            const float dx = (mh.x - sh.x) + (ml.x - sl.x);
            const float dy = (mh.y - sh.y) + (ml.y - sl.y);
            const float dz = (mh.z - sh.z) + (ml.z - sl.z);
            const float h = mh.z + ml.z, s = sh.z + sl.z;
            const float R = (mh.z + sh.z) + (ml.z + sl.z);
            if (!PER) {
                st_pair<GEOM, float>(dx, dy, dz, R, h, s, A, B, sf.x, sf.y, sf.z, ux, uy, uz);
            } else {
                st_images(dx, dy, dz, Lx, Ly, Lz, [&](float qx, float qy, float qz) {
                    st_pair<GEOM, float>(qx, qy, qz, R, h, s, A, B, sf.x, sf.y, sf.z, ux, uy, uz);
                });
            }
        }
        comp_add(sx, ex_, ux);
        comp_add(sy, ey_, uy);
        comp_add(sz, ez_, uz);
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * nt + 3 * (size_t)i;
        o[0] = (double)sx + (double)ex_;
        o[1] = (double)sy + (double)ey_;
        o[2] = (double)sz + (double)ez_;
    }
}

template <int GEOM, bool PER>
__global__ void __launch_bounds__(kStThreads) st_pair_df_kernel(const StRecDF *__restrict__ trg, int nt,
                                                                 const StRecDF *__restrict__ src, int ns, int chunk,
                                                                 StPer P, double *__restrict__ partial)
{
    __shared__ StRecDF tile[kStTile];
    const int i = blockIdx.x * kStThreads + threadIdx.x;
    const bool valid = i < nt;
    const int j0 = blockIdx.y * chunk, j1 = min(ns, j0 + chunk);
    StRecDF me;
    if (valid) {
        me = trg[i];
    } else {
        me.hi = make_float4(0.f, 0.f, 1.0e6f, 1.f);
        me.lo = make_float4(0.f, 0.f, 0.f, 0.f);
        me.fhi = make_float4(0.f, 0.f, 0.f, 1.f);
        me.flo = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const df xi = {me.hi.x, me.lo.x}, yi = {me.hi.y, me.lo.y}, zi = {me.hi.z, me.lo.z};
    const df ra = {me.hi.w, me.lo.w}, ia = {me.fhi.w, me.flo.w};
    const Rad<df> A{ra, ra * ra, ia};
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int t0 = j0; t0 < j1; t0 += kStTile) {
        const int cnt = min(kStTile, j1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kStThreads) tile[k] = src[t0 + k];
        __syncthreads();
        df ux = df_from(0.f), uy = df_from(0.f), uz = df_from(0.f);
        for (int k = 0; k < cnt; ++k) {
            const StRecDF s = tile[k];
            const df xj = {s.hi.x, s.lo.x}, yj = {s.hi.y, s.lo.y}, zj = {s.hi.z, s.lo.z};
            const df rb = {s.hi.w, s.lo.w}, ib = {s.fhi.w, s.flo.w};
            const df fx = {s.fhi.x, s.flo.x}, fy = {s.fhi.y, s.flo.y}, fz = {s.fhi.z, s.flo.z};
            const Rad<df> B{rb, rb * rb, ib};
            const df R = zi + zj;
            if (!PER) {
                st_pair<GEOM, df>(xi - xj, yi - yj, zi - zj, R, zi, zj, A, B, fx, fy, fz, ux, uy, uz);
            } else {
                st_images(to_double(xi - xj), to_double(yi - yj), to_double(zi - zj), P.Lx, P.Ly, P.Lz,
                          [&](double qx, double qy, double qz) {
                              st_pair<GEOM, df>(df_of_double(qx), df_of_double(qy), df_of_double(qz), R, zi, zj, A,
                                                B, fx, fy, fz, ux, uy, uz);
                          });
            }
        }
        ax += to_double(ux);
        ay += to_double(uy);
        az += to_double(uz);
    }
    if (valid) {
        double *o = partial + (size_t)blockIdx.y * 3 * nt + 3 * (size_t)i;
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

// out_t = damp_t / (8 pi eta) sum over chunks (fixed order)
__global__ void st_finalize_kernel(const double *__restrict__ partial, int nchunks, const double *__restrict__ target,
                                   const double *__restrict__ rad_t, double rad_uniform, int nt, double nf, int damp,
                                   double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    double u[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < nchunks; ++s)
        for (int c = 0; c < 3; ++c) u[c] += partial[(size_t)s * 3 * nt + 3 * (size_t)i + c];
    double d = nf;
    if (damp) {
        const double z = target[3 * i + 2], ra = rad_t ? rad_t[i] : rad_uniform;
        if (z < ra) d *= z / ra;
    }
    for (int c = 0; c < 3; ++c) out[3 * i + c] = d * u[c];
}

template <int GEOM, bool PER>
void st_launch(int mode, dim3 grid, cudaStream_t st, const void *trg, int nt, const void *src, int ns, int chunk,
               StPer P, double *partial)
{
    if (mode == RMW_MODE_FP64)
        st_pair_fp64_kernel<GEOM, PER>
            <<<grid, kStThreads, 0, st>>>((const StRecD *)trg, nt, (const StRecD *)src, ns, chunk, P, partial);
    else if (mode == RMW_MODE_DF64)
        st_pair_df_kernel<GEOM, PER>
            <<<grid, kStThreads, 0, st>>>((const StRecDF *)trg, nt, (const StRecDF *)src, ns, chunk, P, partial);
    else
        st_pair_mixed_kernel<GEOM, PER>
            <<<grid, kStThreads, 0, st>>>((const StRecF *)trg, nt, (const StRecF *)src, ns, chunk, P, partial);
}

template <int GEOM>
void st_dispatch(bool per, int mode, dim3 grid, cudaStream_t st, const void *trg, int nt, const void *src, int ns,
                 int chunk, StPer P, double *partial)
{
    if (per) st_launch<GEOM, true>(mode, grid, st, trg, nt, src, ns, chunk, P, partial);
    else st_launch<GEOM, false>(mode, grid, st, trg, nt, src, ns, chunk, P, partial);
}

int check_radii(const double *rad, double uniform, int64_t n, const char *what)
{
    if (n > 0 && !rad && !(uniform > 0)) return fail(RMW_ERR_ARG, std::string(what) + " radius must be positive");
    return RMW_OK;
}

}  // namespace

// u (3 nt) from forces on ns sources; rad_* null means every radius = *_uniform.
int source_target_product(int geom, const double *src, const double *trg, const double *f, const double *rad_s,
                          double rad_s_uniform, const double *rad_t, double rad_t_uniform, int64_t ns, int64_t nt,
                          double eta, const double *L, int mode, double *out, cudaStream_t st)
{
    if (geom != kGeomNoWall && geom != kGeomWall && geom != kGeomFree)
        return fail(RMW_ERR_ARG, "geometry must be RMW_GEOM_NO_WALL, RMW_GEOM_WALL or RMW_GEOM_FREE_SURFACE");
    if (mode != RMW_MODE_FP64 && mode != RMW_MODE_MIXED && mode != RMW_MODE_DF64)
        return fail(RMW_ERR_ARG, "unknown precision mode");
    if (ns < 0 || nt < 0 || ns > (int64_t(1) << 28) || nt > (int64_t(1) << 28))
        return fail(RMW_ERR_ARG, "number of sources or targets out of range [0, 2^28]");
    if ((ns > 0 && (!src || !f)) || (nt > 0 && (!trg || !out))) return fail(RMW_ERR_ARG, "null array pointer");
    if (!(eta > 0)) return fail(RMW_ERR_ARG, "viscosity must be positive");
    if (int rc = check_radii(rad_s, rad_s_uniform, ns, "source")) return rc;
    if (int rc = check_radii(rad_t, rad_t_uniform, nt, "target")) return rc;
    if (nt == 0) return RMW_OK;
    const int NT = (int)nt, NS = (int)ns;
    if (NS == 0) {
        RMW_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 3 * (size_t)NT, st));
        return RMW_OK;
    }
    // enough CTAs for 152 SMs: split the sources when there are few target tiles
    const int ttiles = (NT + kStThreads - 1) / kStThreads;
    const int stiles = (NS + kStTile - 1) / kStTile;
    const int nchunks = std::max(1, std::min(stiles, (4 * 152 + ttiles - 1) / ttiles));
    const size_t rec = (mode == RMW_MODE_FP64) ? sizeof(StRecD) : (mode == RMW_MODE_DF64 ? sizeof(StRecDF)
                                                                                          : sizeof(StRecF));
    const size_t tb = ((rec * (size_t)NT + 255) / 256) * 256, sb = ((rec * (size_t)NS + 255) / 256) * 256;
    void *ws = nullptr;
    if (int rc = scratch(SCRATCH_PAIR, tb + sb + sizeof(double) * 3 * (size_t)NT * nchunks, &ws, st)) return rc;
    void *tp = ws, *sp = (char *)ws + tb;
    double *partial = (double *)((char *)ws + tb + sb);
    const int pb = 256;
    if (mode == RMW_MODE_FP64) {
        st_pack_fp64_kernel<<<(NT + pb - 1) / pb, pb, 0, st>>>(trg, nullptr, rad_t, rad_t_uniform, NT, geom,
                                                              (StRecD *)tp);
        st_pack_fp64_kernel<<<(NS + pb - 1) / pb, pb, 0, st>>>(src, f, rad_s, rad_s_uniform, NS, geom, (StRecD *)sp);
    } else if (mode == RMW_MODE_DF64) {
        st_pack_df_kernel<<<(NT + pb - 1) / pb, pb, 0, st>>>(trg, nullptr, rad_t, rad_t_uniform, NT, geom,
                                                            (StRecDF *)tp);
        st_pack_df_kernel<<<(NS + pb - 1) / pb, pb, 0, st>>>(src, f, rad_s, rad_s_uniform, NS, geom, (StRecDF *)sp);
    } else {
        st_pack_mixed_kernel<<<(NT + pb - 1) / pb, pb, 0, st>>>(trg, nullptr, rad_t, rad_t_uniform, NT, geom,
                                                               (StRecF *)tp);
        st_pack_mixed_kernel<<<(NS + pb - 1) / pb, pb, 0, st>>>(src, f, rad_s, rad_s_uniform, NS, geom,
                                                               (StRecF *)sp);
    }
    const bool per = L && (L[0] > 0 || L[1] > 0 || L[2] > 0);
    const StPer P{L ? L[0] : 0.0, L ? L[1] : 0.0, L ? L[2] : 0.0};
    const int chunk = (NS + nchunks - 1) / nchunks;
    const dim3 grid(ttiles, nchunks);
    if (geom == kGeomWall) st_dispatch<kGeomWall>(per, mode, grid, st, tp, NT, sp, NS, chunk, P, partial);
    else if (geom == kGeomFree) st_dispatch<kGeomFree>(per, mode, grid, st, tp, NT, sp, NS, chunk, P, partial);
    else st_dispatch<kGeomNoWall>(per, mode, grid, st, tp, NT, sp, NS, chunk, P, partial);
    st_finalize_kernel<<<(NT + pb - 1) / pb, pb, 0, st>>>(partial, nchunks, trg, rad_t, rad_t_uniform, NT,
                                                          1.0 / (8.0 * kPi * eta), geom == kGeomWall ? 1 : 0, out);
    RMW_CHECK_LAUNCH("source-target product kernels");
    return RMW_OK;
}

}  // namespace rmw

extern "C" {

// Velocities (3 nt) of targets from forces (3 ns) on sources, per-blob radii;
// geometry RMW_GEOM_NO_WALL / RMW_GEOM_WALL / RMW_GEOM_FREE_SURFACE.
int rmw_source_target_product(int geometry, const double *source, const double *target, const double *force,
                              const double *radius_source, const double *radius_target, int64_t n_source,
                              int64_t n_target, double eta, const double *L_host, int mode, double *out,
                              void *stream)
{
    if ((!radius_source && n_source > 0) || (!radius_target && n_target > 0))
        return rmw::fail(RMW_ERR_ARG, "null radius array");
    return rmw::source_target_product(geometry, source, target, force, radius_source, 0.0, radius_target, 0.0,
                                      n_source, n_target, eta, L_host, mode, out, rmw::as_stream(stream));
}

// Free-surface product of n blobs of radius a: out = M f (3n doubles).
int rmw_free_surface_product(const double *r, const double *force, double *out, int64_t n, double eta, double a,
                             const double *L_host, int mode, void *stream)
{
    return rmw::source_target_product(2, r, r, force, nullptr, a, nullptr, a, n, n, eta, L_host, mode, out,
                                      rmw::as_stream(stream));
}

}  // extern "C"
