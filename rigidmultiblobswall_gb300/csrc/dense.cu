// Dense 3N x 3N translational blob mobility (row-major), FP64:
// * wall = 1: single_wall_fluid_mobility (mobility/mobility.py:1018-1116):
//   B M~(z_eff) B / (8 pi eta a) with the shifted heights and damping;
// * wall = 0: rotne_prager_tensor (mobility/mobility.py:967-1015).
// One thread per 3x3 block; grid.y = target blob, grid.x over source blobs.
#include "mobility_block.cuh"
#include "rmw_common.cuh"

namespace rmw {

namespace {

__global__ void dense_mobility_kernel(const double *__restrict__ r, double *__restrict__ M, int n, double nf,
                                      double a, int wall)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= n) return;
    double blk[3][3], sc;
    uf_block(r, i, j, a, wall != 0, blk, &sc);
    sc *= nf;
    const long long ld = 3LL * n;
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        double *row = M + (3LL * i + u) * ld + 3LL * j;
        row[0] = sc * blk[u][0];
        row[1] = sc * blk[u][1];
        row[2] = sc * blk[u][2];
    }
}

}  // namespace

}  // namespace rmw

extern "C" {

// M (9 n^2 doubles, row-major 3n x 3n) = the dense blob mobility of n blobs.
int rmw_dense_mobility(int wall, const double *r, double *M, int64_t n, double eta, double a, void *stream)
{
    if (n < 0 || n > 65535) return rmw::fail(RMW_ERR_ARG, "number of blobs out of range [0, 65535]");
    if (n > 0 && (!r || !M)) return rmw::fail(RMW_ERR_ARG, "null array pointer");
    if (!(eta > 0) || !(a > 0)) return rmw::fail(RMW_ERR_ARG, "viscosity and blob radius must be positive");
    if (n == 0) return RMW_OK;
    const int N = (int)n, tb = 128;
    rmw::dense_mobility_kernel<<<dim3((N + tb - 1) / tb, N), tb, 0, rmw::as_stream(stream)>>>(
        r, M, N, 1.0 / (8.0 * rmw::kPi * eta * a), a, wall);
    RMW_CHECK_LAUNCH("dense mobility");
    return RMW_OK;
}

}  // extern "C"
