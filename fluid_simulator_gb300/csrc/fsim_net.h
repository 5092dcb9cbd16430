// fsim_net.h -- the pressure warm-start network: kernel launchers (k_conv.cu,
// k_net.cu) and the host-side network object behind the fsim_net_* ABI.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fsim_common.cuh"

// One launch of the tensor-core convolution (forward, or input gradient when
// flip is set and the weights are the per-tap transposed copy).
struct ConvLaunch {
    int taps;                  // 27 (3x3x3, zero padding 1) or 1 (pointwise)
    int n, d, h, w;            // volume
    int cin, cout;             // multiples of 16
    int flip;
    const float* bias;         // or null
    int relu;
    const __nv_bfloat16* mask; // out *= (mask > 0), or null
    int ms, mo;                // mask channel stride / offset
    __nv_bfloat16* y;
    int ys, yo;                // output channel stride / offset
    unsigned* err;
    const CUtensorMap* mx;     // input map (conv_act_map)
    const CUtensorMap* mw;     // weight map (conv_wt_map)
};

struct WgradLaunch {
    int taps, n, d, h, w, cin, cout;
    const __nv_bfloat16* x;    // [vox][cin]
    const __nv_bfloat16* g;    // [vox][cout]
    float* dw;                 // [taps][cout][cin], accumulated
    unsigned* err;
};

bool conv_act_map(CUtensorMap* m, const void* base, int n, int d, int h, int w, int c, int taps);
bool conv_wt_map(CUtensorMap* m, const void* base, int taps, int rows, int kdim, int nt);
int conv_nt(int taps, int cout);
int launch_conv_mma(const ConvLaunch& L, cudaStream_t s);
int launch_conv_wgrad(const WgradLaunch& L, cudaStream_t s);

// ---- the network ------------------------------------------------------------
// Levels 0..3 with 16, 32, 64, 64 channels; two 3x3x3 conv + ReLU per level,
// 2x2x2 stride-2 down-convolutions (space-to-depth + pointwise), trilinear 2x
// up-sampling with skip concatenation, a 1x1x1 head to one channel.
enum { NET_LAYERS = 17, NET_MAX_BATCH = 64 };

struct NetLayer {
    int taps, cin, cout;
    long long w_off, b_off;          // offsets (floats) of weight / bias in the flat parameters
    __nv_bfloat16* wb = nullptr;     // [taps][cout][cin]
    __nv_bfloat16* wt = nullptr;     // [taps][cin][cout]
    CUtensorMap mw, mwt;             // forward / input-gradient weight maps
};

struct NetShape {
    int n = 0, d = 0, h = 0, w = 0;
    bool train = false;
};

struct NetBuf {
    __nv_bfloat16* p = nullptr;
    int c = 0, lev = 0;
};

struct fsim_net {
    cudaStream_t stream = nullptr;
    unsigned* d_err = nullptr;
    NetLayer L[NET_LAYERS];
    long long head_w = 0, head_b = 0;  // head weight (16) and bias offsets
    long long nparams = 0;
    float* theta = nullptr;  // FP32 master parameters
    float* grad = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float out_scale = 1.f;
    long long adam_t = 0;
    __nv_bfloat16* wpool = nullptr;
    // workspace for one shape
    NetShape shape;
    void* ws = nullptr;
    size_t ws_bytes = 0;
    std::vector<NetBuf> act;      // forward tensors
    std::vector<NetBuf> gbuf;     // backward tensors
    std::vector<CUtensorMap> amap;  // activation maps (forward inputs, gradient inputs)
    float* out = nullptr;         // [vox] FP32 prediction
    float* res = nullptr;         // [vox] residual of the prediction (training)
    float* gout = nullptr;        // [vox] loss gradient w.r.t. the prediction (training)
    float* batch_target = nullptr;  // [vox] training batch target (fsim_net_train_batch)
    uint8_t* batch_mask = nullptr;  // [vox] training batch fluid mask
    float loss_l2_weight = 0.1f;    // weight of the relative L2 term of the loss
    double* d_loss = nullptr;     // loss of the last backward pass
    double* d_sums = nullptr;     // per sample: sum r^2, e^2, target^2, b^2
    float* d_coef = nullptr;      // per sample: gradient factors of the two loss terms
    double* d_rms = nullptr;      // solver hook: sum b^2, count
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    long long launches = 0;
};

// forward pass on net->act[X0] (already filled); prediction in net->out
int net_forward(fsim_net* net);
// solver hook: x0 from the solver's rhs/code/flags, forward, guess into `guess`
// (padded grid layout, A' units); returns FSIM_OK or an error code
int net_guess(fsim_net* net, const GridGeom& g, const uint16_t* code, const uint8_t* flags, const double* b,
              float* guess, cudaStream_t s);
