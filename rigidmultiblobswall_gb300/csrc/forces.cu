// Blob forces on the GPU: the right-hand side of the mobility problem.
//
// * blob-blob repulsion (multi_bodies/forces_pycuda.py:40-118, Python form
//   multi_bodies/multi_bodies_functions.py:297-345): from the potential
//   U(r) = U0 exp(-(r - 2a)/b) for r > 2a (linear below), the force on blob i
//   is  f_i = -sum_{j != i} (eps/b) g(r_ij) (r_j - r_i) / r_ij  with
//   g = exp(-(r - 2a)/b) beyond 2a and 1 inside, minimum periodic image.
//   All pairs in FP64, as the reference.  Exact screening: exp(-(r - 2a)/b)
//   is exactly 0 in FP64 once (r - 2a)/b > 746, so such pairs contribute
//   nothing; a conservative FP32 distance test (coordinates relative to the
//   CTA's first target) skips them before any FP64 work.  It is used only
//   where the CTA's spatial extent bounds the FP32 error below the test's
//   margin, so no contributing pair is ever skipped; elsewhere the FP64
//   distance decides.  An optional cutoff restricts the sum to pairs within
//   it (the reference's neighbour-list variant uses 2a + 30 b,
//   multi_bodies/forces_numba.py:228-270).
// * external blob forces (multi_bodies_functions.py:153-189): gravity
//   -g m e_z and the wall repulsion (e/b) exp(-(h - a)/b) (e/b for h <= a).
// The body reduction [F_b, T_b] = K^T f is rmw_rigid_KT_mult.
#include <cmath>

#include "pair_math.cuh"
#include "rmw_common.cuh"

namespace rmw {

namespace {

constexpr int kFThreads = 128;

struct __align__(16) BlobPos {
    double x, y, z, pad;
};

__global__ void __launch_bounds__(kFThreads) blob_blob_kernel(const double *__restrict__ r, double *__restrict__ f,
                                                               int n, double eps_over_b, double inv_b,
                                                               double two_a, double rc, double margin, double Lx,
                                                               double Ly, double Lz, int accumulate)
{
    __shared__ BlobPos tile[kFThreads];
    __shared__ float4 tilef[kFThreads];
    __shared__ double x0[3];
    __shared__ unsigned ext_bits;
    const int i = blockIdx.x * kFThreads + threadIdx.x;
    const bool valid = i < n;
    if (threadIdx.x == 0) {
        const int i0 = blockIdx.x * kFThreads;
        x0[0] = r[3 * i0];
        x0[1] = r[3 * i0 + 1];
        x0[2] = r[3 * i0 + 2];
        ext_bits = 0u;
    }
    __syncthreads();
    const double xi = valid ? r[3 * i] : x0[0], yi = valid ? r[3 * i + 1] : x0[1], zi = valid ? r[3 * i + 2] : x0[2];
    // target coordinates relative to the CTA's first target, in FP32
    const float xf = (float)(xi - x0[0]), yf = (float)(yi - x0[1]), zf = (float)(zi - x0[2]);
    atomicMax(&ext_bits, __float_as_uint(fmaxf(fabsf(xf), fmaxf(fabsf(yf), fabsf(zf)))));
    __syncthreads();
    // FP32 screen only where its error provably stays below the margin:
    // |error of the FP32 distance| <= 2^-22 sqrt(3) (rc + 2 extent + max L)
    const double ext = (double)__uint_as_float(ext_bits);
    const double Lm = fmax(Lx, fmax(Ly, Lz));
    const bool screen32 = 4.2e-7 * (rc + 2.0 * ext + Lm) < margin;
    const float cut2 = (float)((rc + margin) * (rc + margin));
    const float Lxf = (float)Lx, Lyf = (float)Ly, Lzf = (float)Lz;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int t0 = 0; t0 < n; t0 += kFThreads) {
        const int cnt = min(kFThreads, n - t0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const int j = t0 + threadIdx.x;
            const BlobPos p = {r[3 * j], r[3 * j + 1], r[3 * j + 2], 0.0};
            tile[threadIdx.x] = p;
            tilef[threadIdx.x] =
                make_float4((float)(p.x - x0[0]), (float)(p.y - x0[1]), (float)(p.z - x0[2]), 0.f);
        }
        __syncthreads();
        if (!valid) continue;
        for (int k = 0; k < cnt; ++k) {
            const int j = t0 + k;
            if (screen32) {
                const float4 q = tilef[k];
                float ex = q.x - xf, ey = q.y - yf, ez = q.z - zf;
                if (Lxf > 0.f) ex = project(ex, Lxf);
                if (Lyf > 0.f) ey = project(ey, Lyf);
                if (Lzf > 0.f) ez = project(ez, Lzf);
                if (ex * ex + ey * ey + ez * ez >= cut2) continue;
            }
            if (j == i) continue;
            double dx = tile[k].x - xi, dy = tile[k].y - yi, dz = tile[k].z - zi;
            if (Lx > 0) dx = project(dx, Lx);
            if (Ly > 0) dy = project(dy, Ly);
            if (Lz > 0) dz = project(dz, Lz);
            const double rn = sqrt(dx * dx + dy * dy + dz * dz);
            if (!(rn > 0.0) || rn > rc) continue;  // coincident: no direction; beyond rc: exactly zero
            const double g = (rn > two_a) ? exp(-(rn - two_a) * inv_b) : 1.0;
            const double m = eps_over_b * g / rn;
            fx -= m * dx;
            fy -= m * dy;
            fz -= m * dz;
        }
    }
    if (valid) {
        if (accumulate) {
            f[3 * i] += fx;
            f[3 * i + 1] += fy;
            f[3 * i + 2] += fz;
        } else {
            f[3 * i] = fx;
            f[3 * i + 1] = fy;
            f[3 * i + 2] = fz;
        }
    }
}

__global__ void external_force_kernel(const double *__restrict__ r, double *__restrict__ f, int n, double weight,
                                      double blob_radius, double e_over_b, double inv_b, int accumulate)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = r[3 * i + 2];
    const double fz = -weight + ((h > blob_radius) ? e_over_b * exp(-(h - blob_radius) * inv_b) : e_over_b);
    if (accumulate) {
        f[3 * i + 2] += fz;
    } else {
        f[3 * i] = 0.0;
        f[3 * i + 1] = 0.0;
        f[3 * i + 2] = fz;
    }
}

}  // namespace

}  // namespace rmw

extern "C" {

// f (+)= blob-blob repulsion forces of n blobs (device arrays, 3n doubles);
// cutoff <= 0: every pair (exact), else pairs within the cutoff only.
int rmw_blob_blob_forces(const double *r, double *f, int64_t n, double repulsion_strength, double debye_length,
                         double blob_radius, double cutoff, const double *L_host, int accumulate, void *stream)
{
    if (n < 0 || n > (int64_t(1) << 28)) return rmw::fail(RMW_ERR_ARG, "number of blobs out of range [0, 2^28]");
    if (n > 0 && (!r || !f)) return rmw::fail(RMW_ERR_ARG, "null array pointer");
    if (!(debye_length > 0) || !(blob_radius >= 0))
        return rmw::fail(RMW_ERR_ARG, "debye length must be positive and the blob radius non-negative");
    if (n == 0) return RMW_OK;
    const double Lx = L_host ? L_host[0] : 0.0, Ly = L_host ? L_host[1] : 0.0, Lz = L_host ? L_host[2] : 0.0;
    // beyond 2a + 746 b the FP64 exponential is exactly zero: such pairs
    // contribute nothing; a positive cutoff truncates earlier (pairs farther
    // than it are left out, as the reference's neighbour-list variant does);
    // the FP32 screen tests against rc + margin
    const double rexact = 2.0 * blob_radius + 746.0 * debye_length;
    const double rc = (cutoff > 0.0) ? fmin(cutoff, rexact) : rexact;
    const double margin = 1e-3 * rc + 1e-6;
    const int N = (int)n;
    cudaStream_t st = rmw::as_stream(stream);
    rmw::blob_blob_kernel<<<(N + rmw::kFThreads - 1) / rmw::kFThreads, rmw::kFThreads, 0, st>>>(
        r, f, N, repulsion_strength / debye_length, 1.0 / debye_length, 2.0 * blob_radius, rc, margin, Lx, Ly, Lz,
        accumulate);
    RMW_CHECK_LAUNCH("blob-blob forces");
    return RMW_OK;
}

// f (+)= gravity and wall repulsion of n blobs (device arrays, 3n doubles).
int rmw_blob_external_forces(const double *r, double *f, int64_t n, double blob_mass, double blob_radius, double g,
                             double repulsion_strength_wall, double debye_length_wall, int accumulate, void *stream)
{
    if (n < 0 || n > (int64_t(1) << 28)) return rmw::fail(RMW_ERR_ARG, "number of blobs out of range [0, 2^28]");
    if (n > 0 && (!r || !f)) return rmw::fail(RMW_ERR_ARG, "null array pointer");
    if (!(debye_length_wall > 0)) return rmw::fail(RMW_ERR_ARG, "wall debye length must be positive");
    if (n == 0) return RMW_OK;
    const int N = (int)n;
    rmw::external_force_kernel<<<(N + 255) / 256, 256, 0, rmw::as_stream(stream)>>>(
        r, f, N, g * blob_mass, blob_radius, repulsion_strength_wall / debye_length_wall, 1.0 / debye_length_wall,
        accumulate);
    RMW_CHECK_LAUNCH("external blob forces");
    return RMW_OK;
}

}  // extern "C"
