// psf_unet.cuh -- declarations of the learned preconditioner's network (psf_unet.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "pansfem2_gpu.h"

namespace psf {
namespace unet {

typedef __nv_bfloat16 bf16;

constexpr int kLayers = 15, kTensors = 16;
constexpr int kDwSplitMax = 608;

enum ConvMode { kFwdS1 = 0, kFwdS2 = 1, kBwdS1 = 2, kBwdS2 = 3 };

struct LayerDesc {
    int cin, cout, stride, relu, level;
    int in, in_cs, in_c0;
    int out, out_cs, out_c0;
    int woff, boff;
};

int layer_table(int c0, LayerDesc *L);
void tensor_shape(int c0, int *C, int *lev);

// one implicit-GEMM convolution: y[p][c] = act(bias[c] + sum_k A[p][k] B[c][k]),
// A gathered from x by mode (forward stride 1/2, or the transposed forms)
struct ConvArgs {
    const bf16 *x;
    int x_cs, x_c0, cin, hin, win;
    bf16 *y;       // bf16 output, or
    float *y32;    // fp32 output (optionally accumulating)
    int y_cs, y_c0, cstore, accumulate;
    int hout, wout, batch;
    const bf16 *w;        // packed [chunk][kc][N][8]
    const float *bias;    // may be null
    int nchunks, relu, mode;
    int *err;
    const int *skip;      // when non-null and *skip != 0 the launch does nothing
};

struct DwArgs {
    const bf16 *g;
    int gc;
    const bf16 *x;
    int x_cs, x_c0, cin, hin, win;
    int hout, wout, batch, stride, cout;
    long long chunk;
    float *part;
};

cudaError_t launch_conv(int N, const ConvArgs &a, cudaStream_t st);

struct Net {
    int c0 = 16, cap = 1, nparams = 0;
    int H[4] = {0, 0, 0, 0}, W[4] = {0, 0, 0, 0};
    LayerDesc L[kLayers];
    int C[kTensors], lev[kTensors];
    int nchunk_f[kLayers], nchunk_b[kLayers];
    float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    bf16 *wf[kLayers], *wb[kLayers];
    bf16 *t[kTensors];     // activations (t[15] unused: the output is out32)
    float *g[kTensors];    // activation gradients, fp32
    float *out32 = nullptr;
    bf16 *gpre = nullptr;
    float *part = nullptr;
    double *dloss = nullptr;
    int *err = nullptr;
    long long step_count = 0;
    float out_scale = 1.0f;      // the preconditioner multiplies the output by this (set by training)
    cudaStream_t stream = nullptr;
    const int *skip = nullptr;   // forward() launches do nothing while *skip != 0 (graph replays after convergence)
    std::vector<void *> allocs;

    ~Net();
    void release();
    psf_status init(int c0, int H, int W, int batch, uint64_t seed);
    psf_status pack();
    // forward of B samples; input [B][H][W][8] bf16 (null: t[0])
    psf_status forward(int B, const bf16 *input);
    // output gradient from the masked squared error against tgt (fp32 [B][H][W][2])
    // d_rel (may be null) receives the loss relative to that of a zero output
    psf_status loss_grad(int B, const float *tgt, const float *mask, double *d_loss, double *d_rel);
    psf_status backward(int B, const bf16 *input);
    psf_status adam(float lr);
    psf_status check_err();
    psf_status upload_input(int B, const float *host_in);
    size_t npix(int l) const { return (size_t)cap * H[l] * W[l]; }
    size_t npix_b(int B, int l) const { return (size_t)B * H[l] * W[l]; }
};

}  // namespace unet
}  // namespace psf

struct psf_unet {
    psf::unet::Net net;
};
