// Volume spectrum for the projector at power-of-two boxes, sm_103a: the
// reference's pad / sinc^2 / fftshift / rfftn / fftshift (v606:1063-1073)
// computed from the box^3 density without materialising the (2N)^3 padded
// volume, written straight into the blocked copy the slice gather reads.
//
// The padded, fftshifted volume holds the density at signed positions
// j = i - N/2 in [-N/2, N/2) along each axis (mod 2N) and zeros elsewhere.
// A length-2N DFT of such a line splits by output parity k = 2m + e into two
// N-point DFTs of the line's N samples, the odd one premultiplied by
// w^j = exp(-i pi j / N):
//     Y(2m + e) = sum_j [u_j w^{e j}] exp(-2 pi i m j / N).
// Three passes, each a batch of four-step warp FFTs on lines staged in
// shared memory:
//   x: the density rows (sinc^2-weighted on load, as the reference filters
//      the padded volume in float32) -> kx in [0, N], written [z][kx][y];
//   y: lines along y -> ky in [0, 2N), written [ky][kx][z];
//   z: lines along z -> kz in [0, 2N), written in the blocked layout:
//      centred (z, y) order, blocks of 2 (z) x 4 (y) x 2 (x) voxels of 128
//      bytes, x padded to N + 2 (the pad column repeats column N).
// The intermediate arrays (N (N+1) N and 2N (N+1) N complex) stay in L2 at
// box 128.
#include "common.cuh"
#include "warpfft.cuh"

namespace {

constexpr int kVfWarps = 4;  // x and y passes (static shared memory under 48 KB at every box)

// lines of length N a warp transforms at once
template <int N>
__host__ __device__ constexpr int vf_lines() { return 32 / (N / 16); }

// One staged line pair (e = 0, 1) of a length-2N DFT with N nonzero
// samples: line 2q gets u at position (j mod N), line 2q + 1 gets u w^j.
template <int N>
__device__ __forceinline__ void stage_pair(const StageLines<N>& L, int q, int y, float2 u, const float2* tw) {
  const int j = y - N / 2;
  const int n = j & (N - 1);
  L.at(2 * q, n) = u;
  L.at(2 * q + 1, n) = cmul(u, tw_full<-1>(tw, j, 2 * N));
}

// x pass: CTA = one z plane and a band of rows; each warp transforms
// vf_lines/2 rows (two lines per row). Output A1[z][kx][y], kx in [0, N].
template <int N>
__global__ void __launch_bounds__(kVfWarps * 32, 8) vfft_x(const float* __restrict__ vol, float2* __restrict__ a1,
                                                            const float2* __restrict__ tw_g) {
  constexpr int G = vf_lines<N>(), RPW = G / 2, RY = kVfWarps * RPW, m = 2 * N, W = N + 1;
  constexpr int OUTC = RY + 1, RES = (RPW * W + 31) / 32;
  static_assert(W * OUTC <= kVfWarps * G * plane_ld(N), "the output tile fits the staging lines");
  __shared__ float2 s_tw[kMaxFftLen / 2];
  // staging lines; once every warp holds its outputs in registers, the same
  // memory holds the CTA's output tile
  __shared__ float2 s_line[kVfWarps][G * plane_ld(N)];
  float2(*s_out)[OUTC] = reinterpret_cast<float2(*)[OUTC]>(&s_line[0][0]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = blockIdx.y, y0 = blockIdx.x * RY;
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = tw_g[t];
  __syncthreads();
  const StageLines<N> L{s_line[warp]};
  const int half = N / 2;
  const float fz = fftfreq_shifted_f32(z + half, m);
  for (int idx = lane; idx < RPW * N; idx += 32) {
    const int q = idx / N, x = idx - q * N, y = y0 + warp * RPW + q;
    const float fy = fftfreq_shifted_f32(y + half, m), fx = fftfreq_shifted_f32(x + half, m);
    const float w = sinc2_f32(__fmul_rn(fz, fz), __fmul_rn(fy, fy), __fmul_rn(fx, fx));
    const float v = __fmul_rn(__ldg(vol + ((size_t)z * N + y) * N + x), w);
    stage_pair<N>(L, q, x, make_float2(v, 0.f), s_tw);
  }
  __syncwarp();
  warp_fft<N, -1>(L, G, s_tw);
  float2 res[RES];
#pragma unroll
  for (int i = 0; i < RES; ++i) {
    const int idx = lane + 32 * i;
    if (idx < RPW * W) {
      const int q = idx / W, k = idx - q * W;
      res[i] = L.at(2 * q + (k & 1), k >> 1);
    }
  }
  __syncthreads();  // every warp has read its lines
#pragma unroll
  for (int i = 0; i < RES; ++i) {
    const int idx = lane + 32 * i;
    if (idx < RPW * W) {
      const int q = idx / W, k = idx - q * W;
      s_out[k][warp * RPW + q] = res[i];
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < W * RY; idx += blockDim.x) {
    const int k = idx / RY, r = idx - k * RY;
    a1[((size_t)z * W + k) * N + y0 + r] = s_out[k][r];
  }
}

// y pass: CTA = one kx and a band of z; lines along y. Output
// A2[ky][kx][z], ky in [0, 2N) (unshifted).
template <int N>
__global__ void __launch_bounds__(kVfWarps * 32, 8) vfft_y(const float2* __restrict__ a1, float2* __restrict__ a2,
                                                            const float2* __restrict__ tw_g) {
  constexpr int G = vf_lines<N>(), RPW = G / 2, RZ = kVfWarps * RPW, m = 2 * N, W = N + 1;
  constexpr int OUTC = RZ + 1, RES = (RPW * m + 31) / 32;
  constexpr bool kAlias = m * OUTC <= kVfWarps * G * plane_ld(N);  // all boxes but 256
  __shared__ float2 s_tw[kMaxFftLen / 2];
  // staging lines; once every warp holds its outputs in registers, the same
  // memory holds the CTA's output tile (a tile of its own where it does not fit)
  __shared__ float2 s_line[kVfWarps][G * plane_ld(N)];
  __shared__ float2 s_tile[kAlias ? 1 : m][OUTC];
  float2(*s_out)[OUTC] = kAlias ? reinterpret_cast<float2(*)[OUTC]>(&s_line[0][0]) : s_tile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kx = blockIdx.x, z0 = blockIdx.y * RZ;
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = tw_g[t];
  __syncthreads();
  const StageLines<N> L{s_line[warp]};
  for (int idx = lane; idx < RPW * N; idx += 32) {
    const int q = idx / N, y = idx - q * N, z = z0 + warp * RPW + q;
    stage_pair<N>(L, q, y, __ldg(a1 + ((size_t)z * W + kx) * N + y), s_tw);
  }
  __syncwarp();
  warp_fft<N, -1>(L, G, s_tw);
  float2 res[RES];
#pragma unroll
  for (int i = 0; i < RES; ++i) {
    const int idx = lane + 32 * i;
    const int q = idx / m, k = idx - q * m;
    res[i] = L.at(2 * q + (k & 1), k >> 1);
  }
  __syncthreads();  // every warp has read its lines
#pragma unroll
  for (int i = 0; i < RES; ++i) {
    const int idx = lane + 32 * i;
    const int q = idx / m, k = idx - q * m;
    s_out[k][warp * RPW + q] = res[i];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < m * RZ; idx += blockDim.x) {
    const int k = idx / RZ, r = idx - k * RZ;
    a2[((size_t)k * W + kx) * N + z0 + r] = s_out[k][r];
  }
}

// Blocked layout of the slice gather (project.cu): 2 (z) x 4 (y) x 2 (x)
// voxels per 128-byte block, centred (z, y) order, x padded to N + 2.
constexpr int kBZ = 2, kBY = 4, kBX = 2, kBE = kBZ * kBY * kBX;

// z pass: CTA = 4 centred y (one block row) x 2 kx, eight lines along z
// (two FFT lines each), 16 / vf_lines warps of vf_lines FFT lines. Writes
// whole 128-byte blocks of the blocked copy straight from the lines.
template <int N>
__host__ __device__ constexpr int vfz_warps() { return 16 / vf_lines<N>(); }

template <int N>
__global__ void __launch_bounds__(vfz_warps<N>() * 32) vfft_z(const float2* __restrict__ a2,
                                                               float2* __restrict__ blocked,
                                                               const float2* __restrict__ tw_g) {
  constexpr int G = vf_lines<N>(), PPW = G / 2, NW = vfz_warps<N>(), m = 2 * N, W = N + 1, XB = (N + 2) / 2,
                YB = m / kBY;
  static_assert(NW * PPW == 8, "eight (y, x) lines per CTA");
  __shared__ float2 s_tw[kMaxFftLen / 2];
  __shared__ float2 s_line[NW][G * plane_ld(N)];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int yb = blockIdx.y, xb = blockIdx.x;
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = tw_g[t];
  __syncthreads();
  // line l = 4 * (x - 2 xb) + (yc - 4 yb) is pair q = l % PPW of warp l / PPW
  {
    const StageLines<N> L{s_line[warp]};
    for (int idx = lane; idx < PPW * N; idx += 32) {
      const int q = idx / N, z = idx - q * N, l = warp * PPW + q;
      const int yc = kBY * yb + (l & 3), kx = min(kBX * xb + (l >> 2), W - 1);  // the pad column repeats N
      const int ky = yc < N ? yc + N : yc - N;  // centred -> unshifted
      stage_pair<N>(L, q, z, __ldg(a2 + ((size_t)ky * W + kx) * N + z), s_tw);
    }
    __syncwarp();
    warp_fft<N, -1>(L, G, s_tw);
  }
  __syncthreads();
  // block (zb, yb, xb) element ((zc % 2) * 4 + yc % 4) * 2 + x % 2
  for (int idx = threadIdx.x; idx < m * 8; idx += blockDim.x) {
    const int zb = idx / kBE, e = idx - zb * kBE;
    const int zc = kBZ * zb + e / (kBY * kBX), yl = (e / kBX) % kBY, xl = e % kBX;
    const int l = 4 * xl + yl, k = zc < N ? zc + N : zc - N;  // centred -> unshifted kz
    const StageLines<N> L{s_line[l / PPW]};
    blocked[(((size_t)zb * YB + yb) * XB + xb) * kBE + e] = L.at(2 * (l % PPW) + (k & 1), k >> 1);
  }
}

template <int N>
cudaError_t launch_vfft(cudaStream_t st, const float* vol, float2* a1, float2* a2, float2* blocked,
                        const float2* tw) {
  constexpr int G = vf_lines<N>(), RPW = G / 2, R = kVfWarps * RPW;
  static_assert(N % R == 0, "row bands tile the box");
  vfft_x<N><<<dim3(N / R, N), kVfWarps * 32, 0, st>>>(vol, a1, tw);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  vfft_y<N><<<dim3(N + 1, N / R), kVfWarps * 32, 0, st>>>(a1, a2, tw);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  vfft_z<N><<<dim3((N + 2) / 2, 2 * N / 4), vfz_warps<N>() * 32, 0, st>>>(a2, blocked, tw);
  return cudaGetLastError();
}

}  // namespace

// complex elements of the two intermediate arrays (x pass, y pass)
size_t vfft_scratch_elems(int N) { return (size_t)N * (N + 1) * N + (size_t)2 * N * (N + 1) * N; }

cudaError_t launch_volume_spectrum_blocked(cudaStream_t st, const float* vol, int N, float2* scratch,
                                           float2* blocked, const float2* tw) {
  float2* a1 = scratch;
  float2* a2 = scratch + (size_t)N * (N + 1) * N;
  switch (N) {
    case 32: return launch_vfft<32>(st, vol, a1, a2, blocked, tw);
    case 64: return launch_vfft<64>(st, vol, a1, a2, blocked, tw);
    case 128: return launch_vfft<128>(st, vol, a1, a2, blocked, tw);
    case 256: return launch_vfft<256>(st, vol, a1, a2, blocked, tw);
    default: return cudaErrorInvalidValue;
  }
}
