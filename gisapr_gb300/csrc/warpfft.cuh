// Warp-level four-step FFTs on lines staged in shared memory, shared by the
// projector (project.cu) and the volume transform (volfft.cu).
#pragma once

#include "common.cuh"

// Row stride (complex elements) of the padded shared-memory plane: holds the
// N + 1 columns plus one spare slot per 8, chosen by a bank-conflict search.
// Box 256 has no shared-memory plane; its value there is the stride of
// rows_inverse's staging lines (256 elements plus one spare slot per 8).
__host__ __device__ constexpr int plane_ld(int N) {
  return N == 256 ? 290 : (N == 128 ? 150 : (N == 64 ? 74 : 38));
}
__host__ __device__ constexpr int plane_rows(int N) { return N + N / 8; }

// Lines of length N with one spare slot per 8 elements, line stride
// plane_ld(N): element k of line g.
template <int N>
struct StageLines {
  float2* p;
  __device__ __forceinline__ float2& at(int g, int k) const { return p[g * plane_ld(N) + k + (k >> 3)]; }
};

// In-place four-step FFT of ``nlines`` (<= 32 / (N/16)) lines, natural order
// in and out: a 16-point register codelet over n1, twiddles, then N/16-point
// codelets over n2 (N = 16 * (N/16)). One warp, warp barriers only. With
// ``cj`` the input is conjugated on load and the output on store, which
// turns the transform into the one of the opposite direction.
template <int N, int DIR, class Lines>
__device__ __forceinline__ void warp_fft(const Lines& L, int nlines, const float2* tw, bool cj = false) {
  constexpr int L2 = N / 16, G = 32 / L2, T = (G * 16) / 32;
  const int lane = threadIdx.x & 31;
  {
    const int g = lane / L2, n2 = lane % L2;
    if (g < nlines) {
      float2 x[16];
#pragma unroll
      for (int n1 = 0; n1 < 16; ++n1) {
        x[n1] = L.at(g, L2 * n1 + n2);
        if (cj) x[n1].y = -x[n1].y;
      }
      dft<16, DIR>(x);
#pragma unroll
      for (int k1 = 1; k1 < 16; ++k1)
        if (n2) x[k1] = cmul(x[k1], tw_full<DIR>(tw, n2 * k1, N));
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) L.at(g, L2 * k1 + n2) = x[k1];
    }
  }
  __syncwarp();
  float2 y[T][L2];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const int task = lane + 32 * t, g = task / 16, k1 = task % 16;
    if (g < nlines) {
#pragma unroll
      for (int n2 = 0; n2 < L2; ++n2) y[t][n2] = L.at(g, L2 * k1 + n2);
      dft<L2, DIR>(y[t]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const int task = lane + 32 * t, g = task / 16, k1 = task % 16;
    if (g < nlines) {
#pragma unroll
      for (int k2 = 0; k2 < L2; ++k2) L.at(g, k1 + 16 * k2) = cj ? cconj(y[t][k2]) : y[t][k2];
    }
  }
  __syncwarp();
}

