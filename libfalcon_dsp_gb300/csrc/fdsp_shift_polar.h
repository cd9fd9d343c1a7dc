// Launch descriptors of the elementwise stages (NCO shift, polar discriminator).
#pragma once

#include "fdsp_internal.h"

namespace fdsp {

struct ShiftLaunch {
  const float2* in;
  int64_t N;
  int32_t nch;
  int32_t pad_;
  const NcoConst* nco;               // [nch] on the device
  float2* out[kMaxChannels];         // output of each channel
  uint32_t nco_base[kMaxChannels];   // counter of in[0] for each channel (mod R)
};

int launch_freq_shift(const ShiftLaunch& L, cudaStream_t stream);
int launch_polar(const float2* in, int64_t N, float2* d_prev, int start, float* out, cudaStream_t stream);

}  // namespace fdsp
