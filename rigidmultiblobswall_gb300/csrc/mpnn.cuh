// Message-passing network of the near-field preconditioner (mpnn.cu): the
// shared declarations nearfield.cu uses to run it at attach time.
#pragma once
#include <cuda_bf16.h>

#include "../../include/rmw_gb300.h"
#include "rmw_common.cuh"

namespace rmw {

constexpr int kMpIn = 16;       // padded input width (features, edge features)
constexpr int kMpW = 64;        // hidden width
constexpr int kMpOut = 128;     // padded output width
constexpr int kMpTarget = 121;  // 11 x 11 mode coupling
constexpr int kMpSteps = 3;     // message-passing layers
constexpr int kNodeFeat = 2;    // z / R, degree / 8
constexpr int kEdgeFeat = 3;    // horizontal distance, z_dst, z_src (over R)
// normalisation block: node mean, node scale, edge mean, edge scale, target scale
constexpr int kMpNorm = 2 * kNodeFeat + 2 * kEdgeFeat + kMpTarget;

// layers: embed, (msg_t, upd_t) x 3, readout 0..2
constexpr int kMpLayers = 2 + 2 * kMpSteps + 2;
__host__ __device__ constexpr int mp_layer_in(int l)
{
    return l == 0 ? kMpIn : (l <= 2 * kMpSteps ? ((l - 1) % 2 == 0 ? kMpW + kMpIn : 2 * kMpW)
                                               : (l == 2 * kMpSteps + 1 ? 2 * kMpW + kMpIn : kMpW));
}
__host__ __device__ constexpr int mp_layer_out(int l) { return l == kMpLayers - 1 ? kMpOut : kMpW; }
__host__ __device__ constexpr int mp_wofs(int l) { return l == 0 ? 0 : mp_wofs(l - 1) + mp_layer_in(l - 1) * mp_layer_out(l - 1); }
__host__ __device__ constexpr int mp_bofs(int l) { return l == 0 ? 0 : mp_bofs(l - 1) + mp_layer_out(l - 1); }
constexpr int kMpNW = mp_wofs(kMpLayers);
constexpr int kMpNB = mp_bofs(kMpLayers);

struct MpnnNet {
    float *w = nullptr, *b = nullptr;  // FP32 master weights ([out][in] per layer) and biases
    __nv_bfloat16 *wb = nullptr;       // BF16 copy for the tensor cores
    float *adam = nullptr;             // m, v of weights and biases
    float norm[kMpNorm];
    float *dnorm = nullptr;            // device copy of norm
    double cutoff = 0.0;               // learned band reaches up to this centre distance
    double mp_cutoff = 0.0;            // message-passing neighbours below this centre distance
    double radius = 1.0;
    int device = 0;
};

// one graph on the device (see rmw_graph in rmw_gb300.h)
struct MpGraph {
    int n_nodes = 0, n_mp = 0, n_band = 0;
    const float *node_feat = nullptr;   // n_nodes x 2 raw
    const int *mp_src = nullptr, *mp_dst = nullptr, *mp_off = nullptr, *mp_rev = nullptr;
    const float *mp_feat = nullptr;     // n_mp x 3 raw
    const int *band_i = nullptr, *band_j = nullptr, *band_off = nullptr, *band_rev = nullptr;
    const float *band_feat = nullptr;   // n_band x 3 raw
    const float *target = nullptr;      // n_band x 121 raw (pair frame), training only
};

// forward pass: Yf (n_band rows of kMpOut floats, normalised outputs) of graph g
struct MpWork;
int mp_work_create(MpWork **w, int nodes, int mp, int band, cudaStream_t st);
void mp_work_destroy(MpWork *w);
int mp_forward(MpnnNet &net, const MpGraph &g, MpWork &W, cudaStream_t st);
const float *mp_outputs(const MpWork &W);

}  // namespace rmw
