// Double-float helpers for FP64-accurate tall-skinny arithmetic on the FP32 pipe
// (GB300 runs FP64 at ~1/64 of the FP32 rate): an FP64 operand is split once
// into an FP32 pair (hi + lo); products are exact to 2^-48 through fma and sums
// carry a compensation term, which keeps ~44 significant bits.
#pragma once
#include <cuda_runtime.h>

namespace cg {

__device__ __forceinline__ void df_split(double d, float& h, float& l) {
  h = __double2float_rn(d);
  l = __double2float_rn(d - double(h));
}

// (sh, sl) += (ah + al) * (bh + bl), the al * bl term dropped
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float t = sh + p;
  const float bb = t - sh;
  float err = (sh - (t - bb)) + (p - bb);
  err += sl + e;
  sh = t + err;
  sl = err - (sh - t);
}

// (ah, al) + (bh, bl), compensated
__device__ __forceinline__ void df_add(float& h, float& l, float ah, float al, float bh, float bl) {
  const float s = ah + bh;
  const float bb = s - ah;
  float e = (ah - (s - bb)) + (bh - bb);
  e += al + bl;
  h = s + e;
  l = e - (h - s);
}

}  // namespace cg
