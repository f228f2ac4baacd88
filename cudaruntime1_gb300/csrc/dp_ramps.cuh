// dp_ramps.cuh -- a row's band columns as exact integer ramps, shared by the
// anti-diagonal (dp_diag.cu) and lane-per-pair (dp_lane.cu) DP kernels.
#pragma once
#include "tsim_internal.cuh"

namespace tsim {
namespace dp {

// Row band [lo(i), hi(i)] as exact integer ramps,
//   lo(i) = max(0, ceil((a i - Wl) / d)),  hi(i) = min(m - 1, floor((a i + Wh) / d)):
// band: a = m-1, d = n-1, Wl = Wh = w (min(n,m)-1); LCSS window: a = d = 1,
// Wl = Wh = delta; full rows: a = 0, d = 1, Wl = 0, Wh = m-1.  A numerator is
// kept as quotient and remainder by d, so stepping rows costs additions; the
// lo numerator is shifted by K d (K d > Wl) to stay non-negative.
struct Ramp {
  int q, r;
};

struct Ramps {
  int d, K, m, n;
  long long a, Wl, Wh;
  __device__ __forceinline__ Ramp lo_at(long long i) const {
    const long long x = a * i - Wl + (d - 1) + (long long)K * d;
    return Ramp{(int)(x / d), (int)(x % d)};
  }
  __device__ __forceinline__ Ramp hi_at(long long i) const {
    const long long x = a * i + Wh;
    return Ramp{(int)(x / d), (int)(x % d)};
  }
  __device__ __forceinline__ void step(Ramp& x, int dq, int dr) const {
    x.q += dq;
    x.r += dr;
    if (x.r >= d) {
      x.r -= d;
      x.q += 1;
    }
  }
  __device__ __forceinline__ int lo(const Ramp& x) const { return max(0, x.q - K); }
  __device__ __forceinline__ int hi(const Ramp& x) const { return min(m - 1, x.q); }
};

// wd: band width w (DTW/Frechet), window delta (LCSS), < 0 for full rows
__device__ __forceinline__ Ramps make_ramps(int n, int m, int wd, bool lcss) {
  Ramps rp;
  rp.m = m;
  rp.n = n;
  if (wd < 0) {
    rp.a = 0, rp.d = 1, rp.Wl = 0, rp.Wh = m - 1;
  } else if (lcss) {
    rp.a = 1, rp.d = 1, rp.Wl = rp.Wh = wd;
  } else {
    rp.a = m - 1, rp.d = n - 1, rp.Wl = rp.Wh = (long long)wd * (min(n, m) - 1);
  }
  rp.K = (int)(rp.Wl / rp.d) + 1;
  return rp;
}

}  // namespace dp
}  // namespace tsim
