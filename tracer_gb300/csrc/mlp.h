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
  DevBuf img;     // fp16 weights in the MMA layout + fp32 biases
  bool attr_set = false;
};

tr_status guide_reserve(tr_ctx* ctx);
tr_status guide_pack(tr_ctx* ctx);
tr_status guide_forward(tr_ctx* ctx, const float* d_in, int n, float* d_out, __half* d_acts);
void release_guide(tr_ctx* ctx);

}  // namespace trg
