// Launch descriptors of the elementwise stages (NCO shift, polar discriminator).
#pragma once

#include "fdsp_internal.h"

namespace fdsp {

struct ShiftLaunch {
  const float2* in;                  // complex64 input, or complex int16 when i16
  int64_t N;
  int32_t nch;
  int32_t i16;                       // int16 in and out (outputs truncated toward zero)
  const NcoConst* nco;               // [nch] on the device
  float2* out[kMaxChannels];         // output of each channel
  uint32_t nco_base[kMaxChannels];   // counter of in[0] for each channel (mod R)
};

int launch_freq_shift(const ShiftLaunch& L, cudaStream_t stream);
// complex64 -> complex int16 by truncation toward zero (the C++ conversion of
// the reference's int16 overloads)
int launch_cf32_to_ci16(const float2* in, int64_t n, short2* out, cudaStream_t stream);
int launch_polar(const float2* in, int64_t N, float2* d_prev, int start, float* out, cudaStream_t stream);

}  // namespace fdsp
