// mlp.h -- the path-guiding network: sizes, parameter layout, device state.
#pragma once

#include <cuda_fp16.h>

#include "context.h"

namespace trg {
namespace mlp {

constexpr int kIn = 7;       // position in the scene box (3), outgoing direction (3), roughness
constexpr int kInPad = 16;   // one MMA K step
constexpr int kHid = 64;     // four hidden layers
constexpr int kOut = 40;     // 8 lobes x (weight logit, log kappa, mean direction xyz)
constexpr int kOutPad = 48;  // MMA N multiple of 16
constexpr int kLobes = 8;
constexpr int kLayers = 5;
constexpr int kTile = 128;   // rows per MMA (M)
constexpr int kParams = 15592;

}  // namespace mlp

struct GuideModel {
  DevBuf params;  // fp32 master parameters (flat, mlp::param_w / param_b)
  DevBuf img;     // fp16 weights in the forward MMA layout + fp32 biases
  DevBuf img_t;   // fp16 transposed weights of layers 1..4 (backward)
  DevBuf grads, adam_m, adam_v;
  DevBuf acts, out, dout;        // workspace of the unfused entry points (grown on demand)
  DevBuf scal;                   // [1] loss, [2] row scale, [16..] weight partial sums
  DevBuf part;                   // per-CTA gradient partials of the fused training step
  DevBuf losses;                 // per-step batch losses of a training pass
  int64_t step = 0;              // Adam steps taken
  bool attr_set = false;
};

tr_status guide_reserve(tr_ctx* ctx);
tr_status guide_pack(tr_ctx* ctx);
tr_status guide_forward(tr_ctx* ctx, const float* d_in, int n, float* d_out, __half* d_acts);
// Gradient of sum_i dout_i . net(x_i) w.r.t. the parameters into grads (overwritten).
tr_status guide_backward(tr_ctx* ctx, const float* d_in, const float* d_dout, int n, float* d_grads);
// One Adam step on the weighted vMF-mixture NLL of a batch; *d_loss (device) receives the loss.
tr_status guide_train_step(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_w, int n, float lr);
void release_guide(tr_ctx* ctx);
// Forward pass over *d_n rows (a count produced on the device), no host sync;
// each output row is the decoded mixture (kMixFloats floats, mixture.cuh).
tr_status guide_forward_rows_on_device(tr_ctx* ctx, const float* d_in, const unsigned int* d_n, float* d_out);
// `steps` Adam steps on random batches of `batch` rows drawn from `count` records.
tr_status guide_train_on(tr_ctx* ctx, const float* rec_in, const float* rec_dir, const float* rec_w, unsigned int count,
                         int steps, unsigned int batch, float lr, unsigned long long seed, float* mean_loss);

}  // namespace trg
