// Central-slice projector and template tail (v606:856-1147) for sm_103a.
//
// General kernel (boxes 96, 192, 256): one CTA builds one template at a
// time (grid-stride over directions). Every 2-D array of a template lives in
// a global scratch plane owned by the CTA; each pass stages a batch of rows
// or columns in shared memory, transforms it there (block-wide radix-2/3
// FFTs at 96 and 192, four-step warp FFTs at 256) and writes the batch back.
// Boxes 32, 64 and 128 use the shared-memory path further below, which runs
// the same passes on a plane held in shared memory. The passes are:
//
//   A  slice gather + inverse along rows: trilinear samples of the half
//      volume (border clamp, conjugate where the rotated x < 0) feed two
//      N-point inverse FFTs per column (even/odd rows of the 2N grid); the
//      pair combines into exactly the N centred output rows of the 2N-point
//      inverse that the crop keeps (v606:1099-1130). At box 256 (and on the
//      shared-memory path) this pass is its own kernel, rows_inverse.
//   B  C2R along columns (2N-point real output from N+1 coefficients, via an
//      N-point complex inverse), keep the N centred columns, scale 1/(2N)^2;
//      then the forward row FFT that starts the whitening.
//   C  forward column FFT; radial |F| sums per bin (deterministic warp
//      reductions over a host-built bin list).
//   D  divide by the radial mean amplitude (DC bin untouched), inverse
//      column FFT.
//   E  inverse row transform (real part) of pixels centred on the image
//      mean, float32 plane-fit sums (per thread, then a fixed tree).
//   F  plane removal (the least-squares plane in closed form), population
//      sigma normalisation, soft mask, forward row FFT.
//   G  forward column FFT, Fourier crop and packing, FSC weight, L2 norm
//      over the packed half plane, pre-shift (fftshift both dims) into the
//      template bank (v606:1132-1147, 531-537).
//
// The slice coordinates repeat the reference's float32 operations, including
// the rounding of R00*x + R01*y without fused multiply-add: points where that
// sum cancels sit on the conjugation boundary (v606:881-885), and any other
// rounding there picks the mirrored sample.
#include "common.cuh"
#include "warpfft.cuh"

namespace {

struct ProjParams {
  const float2* spectrum;   // cuFFT R2C output [2N][2N][N+1], unshifted
  const float* rot;         // [n_dir][9] float32 rotation matrices (stored transposed)
  const int* dirs;          // directions to build (indices into rot), n_build
  int n_build;
  const float* mask;        // [N][N] or null
  const float* fsc;         // [nb][H] packed FSC
  const int* bin_list;      // [N*(N/2+1)] half-plane indices sorted by radial bin
  const int* bin_ptr;       // [n_bins+1]
  const float* bin_count;   // [n_bins] full-grid counts per bin
  int n_bins;
  const float2* tw;         // twiddles exp(-2 pi i t / kMaxFftLen)
  const float2* tw3;        // twiddles exp(-2 pi i t / kMaxFftLen3) (boxes 3 * 2^k)
  float2* bank;             // [n_dir_out][nb][H] output templates
  const int* out_slot;      // output row in bank for each build index (null => dirs[i])
  float2* scratch;          // per-CTA scratch
  size_t scratch_stride;    // complex elements per CTA
  int* status;              // set to 1 when a plane's bulk-copy wait runs out (or null)
  unsigned wait_limit;      // bound of that wait (attempts)
  const float2* planes;     // pass-A planes written by rows_inverse (or null): [n_build][N][plane_ld(N)]
                            // for the shared-memory path, [n_build][N][N+1] for the general kernel
  int N;
  int nb;
};

constexpr int kThreads = 256;
constexpr int kLineCols = 8;   // columns per batch in pass A
constexpr int kRowBatch = 8;   // rows per batch in passes B/E/F
constexpr int kColBatch = 16;  // columns per batch in passes C/D/G

__device__ __forceinline__ float2 tw_pos(const float2* tw, int num, int den) {
  // exp(+2 pi i num/den) for |num| <= den/2, from the exp(-...) table.
  int t = abs(num) * (kMaxFftLen / den);
  float2 w = tw[t];
  return num >= 0 ? make_float2(w.x, -w.y) : w;
}

// Trilinear sample of the half volume at clamped voxel coordinates, in the
// corner and weight order of grid_sample's 3-D kernel.
__device__ __forceinline__ float2 sample_trilinear(const float2* __restrict__ vol, int m, int w,
                                                   float iz, float iy, float ix) {
  const float fz = floorf(iz), fy = floorf(iy), fx = floorf(ix);
  const int z0 = (int)fz, y0 = (int)fy, x0 = (int)fx;
  const float wz1 = __fsub_rn(iz, fz), wy1 = __fsub_rn(iy, fy), wx1 = __fsub_rn(ix, fx);
  const float wz0 = __fsub_rn(fz + 1.0f, iz), wy0 = __fsub_rn(fy + 1.0f, iy), wx0 = __fsub_rn(fx + 1.0f, ix);
  float2 acc = make_float2(0.f, 0.f);
  // Half-volume storage is unshifted along z and y: stored index = (i + N) mod 2N.
  const int half = m / 2;
#pragma unroll
  for (int dz = 0; dz < 2; ++dz) {
    const int zz = z0 + dz;
    if (zz >= m) continue;
    const float wz = dz ? wz1 : wz0;
    const int zs = (zz + half) % m;
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const int yy = y0 + dy;
      if (yy >= m) continue;
      const float wy = dy ? wy1 : wy0;
      const int ys = (yy + half) % m;
      const float2* row = vol + ((size_t)zs * m + ys) * w;
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const int xx = x0 + dx;
        if (xx >= w) continue;
        const float wx = dx ? wx1 : wx0;
        const float wt = __fmul_rn(__fmul_rn(wx, wy), wz);
        const float2 v = __ldg(row + xx);
        acc.x = __fadd_rn(acc.x, __fmul_rn(v.x, wt));
        acc.y = __fadd_rn(acc.y, __fmul_rn(v.y, wt));
      }
    }
  }
  return acc;
}

// Coordinate of a slice point along one axis, through grid_sample's
// normalise (align_corners=True) and un-normalise, clamped for border mode.
__device__ __forceinline__ float grid_pixel(float c, int size) {
  const float denom = __fsub_rn(__fmul_rn(0.5f, (float)size), 0.5f);
  const float nrm = __fsub_rn(__fdiv_rn(c, denom), 1.0f);
  float pix = __fmul_rn(__fdiv_rn(__fadd_rn(nrm, 1.0f), 2.0f), (float)(size - 1));
  pix = fminf((float)(size - 1), fmaxf(pix, 0.0f));
  return pix;
}

// Hardware square-root approximation (PTX sqrt.approx.f32, relative error
// about 2^-23). Used for the radial |F| sums, whose float32 sums already
// carry larger rounding, and for radial bin indices: rint(sqrt(d2)) of an
// integer d2 <= 2 (N/2)^2 is at least 1/(8 sqrt(d2)) away from a rounding
// boundary, far above the approximation's error, so the bins are exact.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Deterministic float32 block sums over NW warps (xor tree inside each
// warp, warps added in index order). ``scratch`` holds NW entries; two uses
// of the same scratch must be separated by a block barrier.
template <int NW>
__device__ __forceinline__ float4 block_sum_f4(float4 v, float4* scratch) {
  v.x = warp_sum(v.x); v.y = warp_sum(v.y); v.z = warp_sum(v.z); v.w = warp_sum(v.w);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  float4 t = scratch[0];
#pragma unroll
  for (int w = 1; w < NW; ++w) {
    const float4 u = scratch[w];
    t.x += u.x; t.y += u.y; t.z += u.z; t.w += u.w;
  }
  return t;
}
template <int NW>
__device__ __forceinline__ float block_sum_f(float v, float* scratch) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = scratch[0];
#pragma unroll
  for (int w = 1; w < NW; ++w) t += scratch[w];
  return t;
}

// Line batches of the general kernel in shared memory. Box 256 runs its
// 1-D transforms as four-step warp FFTs on padded lines (natural order in
// and out, line stride plane_ld(N), element k at k + k/8), 16 rows per row
// batch; the other boxes use the block-wide radix-2/3 transform on unpadded
// lines, input in fft_in_pos order.
template <int N>
__host__ __device__ constexpr bool warp_lines() { return N == 256; }
template <int N>
__host__ __device__ constexpr int line_len() { return warp_lines<N>() ? plane_ld(N) : N; }
template <int N>
__host__ __device__ constexpr int row_batch() { return warp_lines<N>() ? 16 : kRowBatch; }

// complex elements of the line batches (the largest of passes A-G)
__host__ __device__ constexpr int general_line_elems(int N) {
  const int len = N == 256 ? plane_ld(256) : N;
  const int rb = N == 256 ? 16 : kRowBatch;
  int lines = 2 * kLineCols;
  if (2 * rb > lines) lines = 2 * rb;
  if (kColBatch > lines) lines = kColBatch;
  return lines * len;
}

// position of input element k of a line, and of output element k
template <int N>
__device__ __forceinline__ int lin(int line, int k) {
  return warp_lines<N>() ? line * plane_ld(N) + k + (k >> 3) : line * N + fft_in_pos(k, N);
}
template <int N>
__device__ __forceinline__ int lout(int line, int k) {
  return warp_lines<N>() ? line * plane_ld(N) + k + (k >> 3) : line * N + k;
}

// One warp's transform of one or two lines (``inv``: the unnormalised
// inverse), one out-of-line copy for both directions: inlined at every call
// site of the general kernel, the lane's twiddle factors were hoisted out of
// the pass loops and held in registers throughout (255 registers, spills).
template <int N>
__device__ __noinline__ void warp_fft_lines(float2* p, int nlines, const float2* tw, bool inv) {
  warp_fft<N, -1>(StageLines<N>{p}, nlines, tw, inv);
}

// In-place transforms of ``lines`` lines of the batch (sign -1 forward, +1
// unnormalised inverse), followed by a block barrier.
template <int N>
__device__ __forceinline__ void line_fft(float2* buf, int lines, float sign, const float2* tw,
                                         const float2* tw3) {
  if constexpr (warp_lines<N>()) {
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int g0 = 2 * warp; g0 < lines; g0 += 2 * nw) {
      warp_fft_lines<N>(buf + g0 * plane_ld(N), min(2, lines - g0), tw, sign > 0.f);
    }
    __syncthreads();
  } else {
    smem_fft(buf, N, lines, sign, tw, tw3);
  }
}

template <int N>
__device__ void build_one(const ProjParams& P, int b, int dir, int slot, float2* S, float2* Pk,
                          float2* sm, float4* red4, float* redf, float* s_mu, float* s_div) {
  constexpr int m = 2 * N, W = N + 1, RB = row_batch<N>();
  // unroll of the loops that read the scratch plane: box 256 keeps four
  // loads in flight per thread (the smaller boxes run more CTAs per SM and
  // keep their register count)
  constexpr int UNR = warp_lines<N>() ? 4 : 1;
  const int nb = P.nb, H = nb / 2 + 1;
  const int LDS = N + 1;  // scratch row stride (complex)
  const float* R = P.rot + (size_t)dir * 9;
  const float R00 = R[0], R01 = R[1], R10 = R[3], R11 = R[4], R20 = R[6], R21 = R[7];
  const float inv_m = (float)(1.0 / (double)m);

  // ---- pass A: gather + row inverse (pruned to the N centred rows), unless
  // rows_inverse already wrote this template's plane (P.planes, [N][N+1])
  const float2* A = P.planes != nullptr ? P.planes + (size_t)b * N * LDS : S;
  for (int c0 = 0; P.planes == nullptr && c0 < W; c0 += kLineCols) {
    const int nc = min(kLineCols, W - c0);
    const int total = nc * m;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int cl = t / m, r = t - cl * m;  // r: standard-order row of the 2N grid
      const int c = c0 + cl;
      const int kys = (r + N) % m;            // row in the shifted base grid
      const float gy = __fmul_rn((float)(kys - N), inv_m);
      const float gx = __fmul_rn((float)c, inv_m);
      float rx = __fadd_rn(__fmul_rn(R00, gx), __fmul_rn(R01, gy));
      float ry = __fadd_rn(__fmul_rn(R10, gx), __fmul_rn(R11, gy));
      float rz = __fadd_rn(__fmul_rn(R20, gx), __fmul_rn(R21, gy));
      const bool conj = rx < 0.0f;
      if (conj) { rx = -rx; ry = -ry; rz = -rz; }
      const float cz = __fadd_rn(__fmul_rn(rz, (float)m), (float)(m / 2));
      const float cy = __fadd_rn(__fmul_rn(ry, (float)m), (float)(m / 2));
      const float cx = __fmul_rn(rx, (float)m);
      float2 v = sample_trilinear(P.spectrum, m, W, grid_pixel(cz, m), grid_pixel(cy, m),
                                  grid_pixel(cx, W));
      if (conj) v.y = -v.y;
      const int e = r & 1, q = r >> 1;
      sm[lin<N>(cl * 2 + e, q)] = v;
    }
    __syncthreads();
    line_fft<N>(sm, 2 * nc, +1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int cl = t / N, i = t - cl * N;
      const int u = i - N / 2;               // signed output row of the 2N-point inverse
      const int k = (u + N) % N;
      const float2 a0 = sm[lout<N>(cl * 2, k)];
      const float2 a1 = sm[lout<N>(cl * 2 + 1, k)];
      const float2 z = cadd(a0, cmul(tw_pos_any(P.tw, P.tw3, u, m), a1));
      S[(size_t)i * LDS + c0 + cl] = z;
    }
    __syncthreads();
  }

  // ---- pass B: C2R along columns, keep centred N, then forward row FFT
  const float scale_b = (float)(1.0 / ((double)m * (double)m));
  float2* sm2 = sm + RB * line_len<N>();
  for (int i0 = 0; i0 < N; i0 += RB) {
    const int nr = min(RB, N - i0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
      const int rl = t / N, k = t - rl * N;
      const float2* Z = A + (size_t)(i0 + rl) * LDS;
      float2 ye, yo;
      if (k == 0) {
        const float a = Z[0].x, b = Z[N].x;
        ye = make_float2(a + b, 0.f);
        yo = make_float2(a - b, 0.f);
      } else {
        const float2 zk = Z[k], zc = cconj(Z[N - k]);
        ye = cadd(zk, zc);
        yo = cmul(csub(zk, zc), tw_pos_any(P.tw, P.tw3, k, m));
      }
      // W = Ye + i*Yo
      sm[lin<N>(rl, k)] = make_float2(ye.x - yo.y, ye.y + yo.x);
    }
    __syncthreads();
    line_fft<N>(sm, nr, +1.0f, P.tw, P.tw3);
    // p(2n) = Re z(n), p(2n+1) = Im z(n); keep v = (j - N/2) mod 2N.
    for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
      const int rl = t / N, j = t - rl * N;
      const int v = (j - N / 2 + m) % m;
      const float2 zz = sm[lout<N>(rl, v >> 1)];
      const float p = ((v & 1) ? zz.y : zz.x) * scale_b;
      sm2[lin<N>(rl, j)] = make_float2(p, 0.f);
    }
    __syncthreads();
    line_fft<N>(sm2, nr, -1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nr * (N / 2 + 1); t += blockDim.x) {
      const int rl = t / (N / 2 + 1), k = t - rl * (N / 2 + 1);
      S[(size_t)(i0 + rl) * LDS + k] = sm2[lout<N>(rl, k)];
    }
    __syncthreads();
  }

  // ---- pass C: forward column FFT (kx in [0, N/2])
  const int HC = N / 2 + 1;
  for (int c0 = 0; c0 < HC; c0 += kColBatch) {
    const int nc = min(kColBatch, HC - c0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      sm[lin<N>(cl, r)] = S[(size_t)r * LDS + c0 + cl];
    }
    __syncthreads();
    line_fft<N>(sm, nc, -1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      S[(size_t)r * LDS + c0 + cl] = sm[lout<N>(cl, r)];
    }
    __syncthreads();
  }
  // radial sums of |F| over the full grid in float32 (columns 1..N/2-1
  // stand for two bins): per lane, then a fixed xor tree across the warp
  {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int b = warp; b < P.n_bins; b += nw) {
      float acc = 0.f;
#pragma unroll (UNR / 2 > 0 ? UNR / 2 : 1)
      for (int e = P.bin_ptr[b] + lane; e < P.bin_ptr[b + 1]; e += 32) {
        const int idx = P.bin_list[e];
        const int r = idx / HC, kx = idx - r * HC;
        const float2 f = S[(size_t)r * LDS + kx];
        const float a = sqrt_approx(fmaf(f.x, f.x, f.y * f.y));
        acc += (kx == 0 || kx == N / 2) ? a : 2.0f * a;
      }
      acc = warp_sum(acc);
      if (lane == 0) s_div[b] = (b == 0) ? 1.0f : __fdiv_rn(P.bin_count[b], acc);
    }
  }
  // The DC term (bin 0, left as it is) over N^2 is the image mean; it is read
  // before column 0 is transformed and taken out of every pixel in pass E,
  // so the float32 plane-fit and variance sums run on centred values.
  const float scale_e = (float)(1.0 / ((double)N * (double)N));
  if (threadIdx.x == 0) s_mu[0] = S[0].x * scale_e;
  __syncthreads();

  // ---- pass D: scale by the radial divisor, inverse column FFT
  for (int c0 = 0; c0 < HC; c0 += kColBatch) {
    const int nc = min(kColBatch, HC - c0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      const int kx = c0 + cl;
      const int ky = r < N / 2 ? r : r - N;
      const int bin = (int)rintf(sqrtf((float)(ky * ky + kx * kx)));
      sm[lin<N>(cl, r)] = cscale(S[(size_t)r * LDS + kx], s_div[bin]);
    }
    __syncthreads();
    line_fft<N>(sm, nc, +1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      S[(size_t)r * LDS + c0 + cl] = sm[lout<N>(cl, r)];
    }
    __syncthreads();
  }

  // ---- pass E: inverse row transform (real part), centred pixels, float32
  // plane-fit sums (per thread, then a fixed tree across the block)
  const float mu = s_mu[0];
  float fz = 0.f, fxz = 0.f, fyz = 0.f, fww = 0.f;
  for (int i0 = 0; i0 < N; i0 += RB) {
    const int nr = min(RB, N - i0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
      const int rl = t / N, k = t - rl * N;
      const float2* G = S + (size_t)(i0 + rl) * LDS;
      float2 y;
      if (k == 0 || k == N / 2) y = make_float2(G[k].x, 0.f);
      else if (k < N / 2) y = G[k];
      else y = cconj(G[N - k]);
      sm[lin<N>(rl, k)] = y;
    }
    __syncthreads();
    line_fft<N>(sm, nr, +1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
      const int rl = t / N, j = t - rl * N;
      const int i = i0 + rl;
      const float w = fmaf(sm[lout<N>(rl, j)].x, scale_e, -mu);
      S[(size_t)i * LDS + j] = make_float2(w, 0.f);
      fz += w;
      fxz = fmaf((float)i, w, fxz);
      fyz = fmaf((float)j, w, fyz);
      fww = fmaf(w, w, fww);
    }
    __syncthreads();
  }
  // Least-squares plane z = c0*row + c1*col + c2 over the full N x N grid in
  // closed form: the grid is a Cartesian product, so the centred row and
  // column coordinates are orthogonal and the 3x3 normal equations decouple.
  const float4 s4 = block_sum_f4<kThreads / 32>(make_float4(fz, fxz, fyz, fww), red4);
  constexpr float kMid = 0.5f * (float)(N - 1);
  constexpr float kSii = (float)((double)N * (double)N * ((double)N * (double)N - 1.0) / 12.0);
  const float pc0 = (s4.y - kMid * s4.x) / kSii;
  const float pc1 = (s4.z - kMid * s4.x) / kSii;
  const float pcm = s4.x * scale_e - (pc0 + pc1) * kMid;
  // Residual energy sum (w - P)^2 = sum w^2 - sum P w (the residual of a
  // least-squares fit is orthogonal to the fit); where the plane holds most
  // of the energy the subtraction would cancel, and the residual is summed
  // directly instead (a block-uniform choice).
  float ssr = s4.w - fmaf(pc0, s4.y, fmaf(pc1, s4.z, pcm * s4.x));
  if (!(ssr > 0.25f * s4.w)) {
    float fsv = 0.f;
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int i = t / N, j = t - i * N;
      const float v = S[(size_t)i * LDS + j].x - fmaf(pc0, (float)i, fmaf(pc1, (float)j, pcm));
      fsv = fmaf(v, v, fsv);
    }
    ssr = block_sum_f<kThreads / 32>(fsv, redf);
  }
  const float sd = sqrtf(ssr * scale_e);
  const float inv_sd = sd > 1e-12f ? 1.0f / sd : 1.0f;

  // ---- pass F: normalise, mask, forward row FFT
  for (int i0 = 0; i0 < N; i0 += RB) {
    const int nr = min(RB, N - i0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
      const int rl = t / N, j = t - rl * N;
      const int i = i0 + rl;
      float f = (S[(size_t)i * LDS + j].x - fmaf(pc0, (float)i, fmaf(pc1, (float)j, pcm))) * inv_sd;
      if (P.mask != nullptr) f *= P.mask[(size_t)i * N + j];
      sm[lin<N>(rl, j)] = make_float2(f, 0.f);
    }
    __syncthreads();
    line_fft<N>(sm, nr, -1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nr * HC; t += blockDim.x) {
      const int rl = t / HC, k = t - rl * HC;
      S[(size_t)(i0 + rl) * LDS + k] = sm[lout<N>(rl, k)];
    }
    __syncthreads();
  }
  // ---- pass G: forward column FFT
  for (int c0 = 0; c0 < HC; c0 += kColBatch) {
    const int nc = min(kColBatch, HC - c0);
#pragma unroll (UNR)
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      sm[lin<N>(cl, r)] = S[(size_t)r * LDS + c0 + cl];
    }
    __syncthreads();
    line_fft<N>(sm, nc, -1.0f, P.tw, P.tw3);
    for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
      const int r = t / nc, cl = t - r * nc;
      S[(size_t)r * LDS + c0 + cl] = sm[lout<N>(cl, r)];
    }
    __syncthreads();
  }
  // crop + pack + FSC, L2 norm (float32 per thread, fixed tree across the block)
  float fss = 0.f;
#pragma unroll (UNR)
  for (int t = threadIdx.x; t < nb * H; t += blockDim.x) {
    const int r = t / H, c = t - r * H;
    const int ky = r < nb / 2 ? r : r - nb;
    float2 f;
    if (c < nb / 2) {
      f = S[(size_t)((ky + N) % N) * LDS + c];
    } else if (nb == N) {
      f = S[(size_t)((ky + N) % N) * LDS + N / 2];
    } else {
      f = cconj(S[(size_t)((-ky + N) % N) * LDS + nb / 2]);
    }
    f = cscale(f, P.fsc[t]);
    Pk[t] = f;
    fss = fmaf(f.x, f.x, fmaf(f.y, f.y, fss));
  }
  const float inv_norm = 1.0f / sqrtf(block_sum_f<kThreads / 32>(fss, redf));
  float2* out = P.bank + (size_t)slot * nb * H;
  for (int t = threadIdx.x; t < nb * H; t += blockDim.x) {
    const int r = t / H, c = t - r * H;
    const int rs = (r + nb / 2) % nb, cs = (c + H / 2) % H;
    out[(size_t)rs * H + cs] = cscale(Pk[t], inv_norm);
  }
  __syncthreads();
}

// Box 256 asks for two CTAs per SM (128 registers); a minimum of 0 leaves the
// other boxes to the compiler's default (40 registers; 72 with a minimum of 1).
template <int N>
__global__ void __launch_bounds__(kThreads, warp_lines<N>() ? 2 : 0) project_templates(ProjParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  float2* s_tw = sm + general_line_elems(N);
  float4* red4 = reinterpret_cast<float4*>(s_tw + kMaxFftLen / 2);  // [kThreads / 32]
  float* redf = reinterpret_cast<float*>(red4 + kThreads / 32);      // [kThreads / 32]
  float* s_mu = redf + kThreads / 32;                                 // [4]
  float* s_div = s_mu + 4;                                            // [n_bins + 4]
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = P.tw[t];
  __syncthreads();
  ProjParams Q = P;
  Q.tw = s_tw;
  float2* S = P.scratch + (size_t)blockIdx.x * P.scratch_stride;
  float2* Pk = S + (size_t)N * (N + 1);
  for (int b = blockIdx.x; b < P.n_build; b += gridDim.x) {
    const int dir = P.dirs[b];
    const int slot = P.out_slot ? P.out_slot[b] : dir;
    build_one<N>(Q, b, dir, slot, S, Pk, sm, red4, redf, s_mu, s_div);
  }
}

}  // namespace

// complex elements of the pass-A planes of n_build templates (shared-memory
// path, N <= 128): N rows of plane_ld(N) each
size_t project_slice_elems(int N, int n_build) {
  return (size_t)n_build * N * (N == 128 ? 150 : (N == 64 ? 74 : 38));
}

size_t project_scratch_elems(int N, int nb) {
  return (size_t)N * (N + 1) + (size_t)nb * (nb / 2 + 1);
}

size_t project_smem_bytes(int N, int n_bins) {
  return (size_t)general_line_elems(N) * sizeof(float2) + (kMaxFftLen / 2) * sizeof(float2) +
         (kThreads / 32) * (sizeof(float4) + sizeof(float)) + (size_t)(4 + n_bins + 4) * sizeof(float);
}

template <int N>
static cudaError_t launch_general(const ProjParams& P, int grid, size_t smem, cudaStream_t st) {
  static size_t set_smem = 0;  // attribute set once per size, never inside a stream capture
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(project_templates<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  project_templates<N><<<grid, kThreads, smem, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_project_templates(cudaStream_t st, const float2* spectrum, const float* rot,
                                     const int* dirs, int n_build, const int* out_slot,
                                     const float* mask, const float* fsc, const int* bin_list,
                                     const int* bin_ptr, const float* bin_count, int n_bins,
                                     const float2* tw, const float2* tw3, float2* bank, float2* scratch,
                                     int grid, int N, int nb) {
  if (n_build <= 0) return cudaSuccess;
  ProjParams P;
  P.status = nullptr; P.wait_limit = 0;
  P.spectrum = spectrum; P.rot = rot; P.dirs = dirs; P.n_build = n_build; P.mask = mask;
  P.fsc = fsc; P.bin_list = bin_list; P.bin_ptr = bin_ptr; P.bin_count = bin_count;
  P.n_bins = n_bins; P.tw = tw; P.tw3 = tw3; P.bank = bank; P.out_slot = out_slot; P.scratch = scratch; P.planes = nullptr;
  P.scratch_stride = project_scratch_elems(N, nb); P.N = N; P.nb = nb;
  const size_t smem = project_smem_bytes(N, n_bins);
  switch (N) {
    case 96: return launch_general<96>(P, grid, smem, st);
    case 192: return launch_general<192>(P, grid, smem, st);
    // powers of two up to 128 take the shared-memory path, box 256
    // launch_project_templates_planes
    default: return cudaErrorInvalidValue;
  }
}

// ===========================================================================
// Shared-memory projector for boxes 32, 64 and 128, in three launches:
// spectrum_blocked (a blocked copy of the half-volume spectrum),
// rows_inverse (slice gather and pass A at high occupancy, each template's
// plane written to global memory) and project_templates_smem (passes B-G,
// one template at a time per CTA, its plane arriving by bulk async copies).
//
// The template's working set (the N x (N+1) plane left by the pruned
// inverse along rows, then the N x (N/2+1) spectra of the whitening) stays in
// shared memory. Every 1-D transform is a four-step 16 x (N/16) FFT done by
// one warp on whole lines: a 16-point register codelet over n1, twiddles,
// then N/16-point codelets, with only warp barriers inside a pass and block
// barriers between passes. The passes compute what the general kernel above
// computes (same float32 slice coordinates); the forward transforms of real
// rows run two rows per complex line, and the block sums are float32 over a
// fixed tree.
// ===========================================================================
namespace {

// Warps of the template-tail CTA (a template parameter of the kernel; the
// shared-memory scratch of the block sums is sized for the largest count)
constexpr int kSmemMaxWarps = 20;

// Columns a warp transforms per pass-A round: G = 32 / (N/16) lines, two
// per column (even and odd rows of the 2N grid). The even line of column c
// is transformed in place in plane column c (which then receives the
// column's output); only the odd lines need staging.
template <int N>
__host__ __device__ constexpr int pass_a_cols() { return 16 / (N / 16); }




// The half-volume spectrum in the blocked layout the slice gather reads:
// centred order along z and y, cut into blocks of 2 (z) x 4 (y) x 2 (x)
// voxels, one 128-byte line each (x padded to an even count). A trilinear
// footprint then spans about two lines instead of four rows, and the 32
// samples of one warp load touch 12 lines instead of 21 (counted for
// random orientations), which is what bounds the gather's L1 throughput.
constexpr int kBZ = 2, kBY = 4, kBX = 2, kBE = kBZ * kBY * kBX;

template <int N>
__host__ __device__ constexpr int blocked_x() { return (N + 1 + kBX - 1) / kBX; }

template <int N>
__device__ __forceinline__ int blocked_off(int z, int y, int x) {
  constexpr int YB = 2 * N / kBY, XB = blocked_x<N>();
  return (((z / kBZ) * YB + y / kBY) * XB + x / kBX) * kBE + ((z % kBZ) * kBY + y % kBY) * kBX + x % kBX;
}

template <int N>
__global__ void __launch_bounds__(256) spectrum_blocked(const float2* __restrict__ spectrum,
                                                        float2* __restrict__ out) {
  constexpr int m = 2 * N, W = N + 1, XB = blocked_x<N>(), YB = m / kBY;
  const int total = (m / kBZ) * YB * XB * kBE;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < total; o += gridDim.x * blockDim.x) {
    const int e = o % kBE, blk = o / kBE;
    const int xb = blk % XB, yb = (blk / XB) % YB, zb = blk / (XB * YB);
    const int x = xb * kBX + e % kBX, y = yb * kBY + (e / kBX) % kBY, z = zb * kBZ + e / (kBX * kBY);
    // the spectrum is stored unshifted along z and y: index (i + N) mod 2N
    const int zs = z < N ? z + N : z - N, ys = y < N ? y + N : y - N;
    out[o] = __ldg(spectrum + ((size_t)zs * m + ys) * W + min(x, W - 1));
  }
}

// Trilinear sample at the slice point's voxel coordinates (grid_sample's
// normalise/un-normalise pair with align_corners=True is the identity, so
// the coordinates are used directly, clamped for border padding). Corners
// past the last voxel carry weight 0 and are read clamped. ``vol`` is the
// blocked copy written by spectrum_blocked.
template <int N>
__device__ __forceinline__ float2 sample_slice(const float2* __restrict__ vol, float cz, float cy, float cx) {
  constexpr int m = 2 * N, W = N + 1;
  const float pz = fminf((float)(m - 1), fmaxf(cz, 0.0f));
  const float py = fminf((float)(m - 1), fmaxf(cy, 0.0f));
  const float px = fminf((float)(W - 1), fmaxf(cx, 0.0f));
  const float fz = floorf(pz), fy = floorf(py), fx = floorf(px);
  const int z0 = (int)fz, y0 = (int)fy, x0 = (int)fx;
  const int z1 = min(z0 + 1, m - 1), y1 = min(y0 + 1, m - 1), x1 = min(x0 + 1, W - 1);
  const float wz1 = __fsub_rn(pz, fz), wy1 = __fsub_rn(py, fy), wx1 = __fsub_rn(px, fx);
  const float wz0 = __fsub_rn(fz + 1.0f, pz), wy0 = __fsub_rn(fy + 1.0f, py), wx0 = __fsub_rn(fx + 1.0f, px);
  const float2 v000 = __ldg(vol + blocked_off<N>(z0, y0, x0)), v001 = __ldg(vol + blocked_off<N>(z0, y0, x1));
  const float2 v010 = __ldg(vol + blocked_off<N>(z0, y1, x0)), v011 = __ldg(vol + blocked_off<N>(z0, y1, x1));
  const float2 v100 = __ldg(vol + blocked_off<N>(z1, y0, x0)), v101 = __ldg(vol + blocked_off<N>(z1, y0, x1));
  const float2 v110 = __ldg(vol + blocked_off<N>(z1, y1, x0)), v111 = __ldg(vol + blocked_off<N>(z1, y1, x1));
  const float w000 = __fmul_rn(__fmul_rn(wx0, wy0), wz0), w001 = __fmul_rn(__fmul_rn(wx1, wy0), wz0);
  const float w010 = __fmul_rn(__fmul_rn(wx0, wy1), wz0), w011 = __fmul_rn(__fmul_rn(wx1, wy1), wz0);
  const float w100 = __fmul_rn(__fmul_rn(wx0, wy0), wz1), w101 = __fmul_rn(__fmul_rn(wx1, wy0), wz1);
  const float w110 = __fmul_rn(__fmul_rn(wx0, wy1), wz1), w111 = __fmul_rn(__fmul_rn(wx1, wy1), wz1);
  float2 a;
  a.x = v000.x * w000; a.y = v000.y * w000;
  a.x = fmaf(v001.x, w001, a.x); a.y = fmaf(v001.y, w001, a.y);
  a.x = fmaf(v010.x, w010, a.x); a.y = fmaf(v010.y, w010, a.y);
  a.x = fmaf(v011.x, w011, a.x); a.y = fmaf(v011.y, w011, a.y);
  a.x = fmaf(v100.x, w100, a.x); a.y = fmaf(v100.y, w100, a.y);
  a.x = fmaf(v101.x, w101, a.x); a.y = fmaf(v101.y, w101, a.y);
  a.x = fmaf(v110.x, w110, a.x); a.y = fmaf(v110.y, w110, a.y);
  a.x = fmaf(v111.x, w111, a.x); a.y = fmaf(v111.y, w111, a.y);
  return a;
}

// Padded plane layout: one spare slot after every 8 elements along both rows
// and columns, row stride plane_ld(N). With it the four-step loads and stores
// of row and column passes touch each 8-byte bank at most twice (three times
// for two of the six patterns) per warp access.

template <int N>
struct Plane {
  float2* p;
  __device__ __forceinline__ int off(int r, int c) const { return (r + (r >> 3)) * plane_ld(N) + c + (c >> 3); }
  __device__ __forceinline__ float2& operator()(int r, int c) const { return p[off(r, c)]; }
};

// Line accessors for warp_fft: element k of line g.
template <int N>
struct RowLines {  // lines are plane rows r0 + g
  Plane<N> pl; int r0;
  __device__ __forceinline__ float2& at(int g, int k) const { return pl(r0 + g, k); }
};
template <int N>
struct ColLines {  // lines are plane columns c0 + g
  Plane<N> pl; int c0;
  __device__ __forceinline__ float2& at(int g, int k) const { return pl(k, c0 + g); }
};

// The value of the central slice at row r (standard order of the 2N grid)
// and column c: the reference's float32 coordinates, border-clamped
// trilinear sample, conjugated where the rotated x is negative.
template <int N>
__device__ __forceinline__ float2 slice_value(const float2* __restrict__ spectrum, const float* __restrict__ R,
                                              int r, int c) {
  constexpr int m = 2 * N;
  const float inv_m = (float)(1.0 / (double)m);
  const int kys = (r + N) % m;
  const float gy = __fmul_rn((float)(kys - N), inv_m);
  const float gx = __fmul_rn((float)c, inv_m);
  float rx = __fadd_rn(__fmul_rn(R[0], gx), __fmul_rn(R[1], gy));
  float ry = __fadd_rn(__fmul_rn(R[3], gx), __fmul_rn(R[4], gy));
  float rz = __fadd_rn(__fmul_rn(R[6], gx), __fmul_rn(R[7], gy));
  const bool conj = rx < 0.0f;
  if (conj) { rx = -rx; ry = -ry; rz = -rz; }
  const float cz = __fadd_rn(__fmul_rn(rz, (float)m), (float)(m / 2));
  const float cy = __fadd_rn(__fmul_rn(ry, (float)m), (float)(m / 2));
  const float cx = __fmul_rn(rx, (float)m);
  float2 v = sample_slice<N>(spectrum, cz, cy, cx);
  if (conj) v.y = -v.y;
  return v;
}


// Lines of the paired row passes: line q is plane row r0 + 2q, which holds
// z = a + i b for the real rows a = r0 + 2q and b = r0 + 2q + 1.
template <int N>
struct PairLines {
  Plane<N> pl; int r0;
  __device__ __forceinline__ float2& at(int g, int k) const { return pl(r0 + 2 * g, k); }
};

// After a forward FFT of the paired lines of rows r0 .. r0 + 2G - 1, split
// each line into the half spectra of its two real rows (k in [0, N/2]):
// A(k) = (Z(k) + conj Z(N-k)) / 2 into the first row, B(k) = (Z(k) -
// conj Z(N-k)) / 2i into the second. A task (q, k) reads positions k and
// N-k of its line and writes position k of both rows; no other task reads
// those, so the split runs in place without a barrier.
template <int N>
__device__ __forceinline__ void pair_split(const Plane<N>& Z, int r0, int lane) {
  constexpr int HC = N / 2 + 1, G = 32 / (N / 16);
  for (int idx = lane; idx < G * HC; idx += 32) {
    const int q = idx / HC, k = idx - q * HC;
    const int i1 = r0 + 2 * q;
    const float2 zk = Z(i1, k), zn = Z(i1, (N - k) & (N - 1));
    Z(i1, k) = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    Z(i1 + 1, k) = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
  }
}


// The pass-A plane of one template arrives by bulk async copies: 8 plane
// rows per copy (the rows of one padding group are contiguous in shared
// memory), completion counted on one mbarrier. Every wait is bounded.
constexpr unsigned kPlaneWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int N>
__device__ __forceinline__ void plane_load(float2* Zs, const float2* src, uint64_t* bar) {
  constexpr uint32_t kChunk = 8u * plane_ld(N) * sizeof(float2);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(kChunk * (N / 8)) : "memory");
  for (int q = 0; q < N / 8; ++q)
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(Zs + 9 * q * plane_ld(N))),
        "l"(src + (size_t)8 * q * plane_ld(N)), "r"(kChunk), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool plane_wait(uint64_t* bar, uint32_t parity, unsigned limit) {
  for (unsigned i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <int N, int kSmemWarps>
__device__ void build_one_smem(const ProjParams& P, int slot, float2* Zs, const float2* tw, float* s_div,
                               float4* red4, float* red, float* s_misc, const unsigned short* s_bins,
                               const int* s_bptr, const float* s_fsc, const float2* next_plane, uint64_t* bar) {
  constexpr int HC = N / 2 + 1, L2 = N / 16, G = 32 / L2, RP = 2 * G;
  constexpr int kSmemThreads = 32 * kSmemWarps;
  const Plane<N> Z{Zs};
  const int nb = P.nb, H = nb / 2 + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // ---- pass B: C2R along rows (the plane written by rows_inverse arrived by
  // bulk copy before this call), keep the centred N columns as real values
  constexpr int m = 2 * N;
  const float scale_b = (float)(1.0 / ((double)m * (double)m));
  for (int r0 = warp * G; r0 < N; r0 += kSmemWarps * G) {
    const RowLines<N> RL{Z, r0};
    // W = Ye + i Yo. A lane owns the pair (k, N-k): both outputs depend on
    // Z_k and Z_{N-k} only, so the rows are rewritten in place.
    for (int idx = lane; idx < G * (N / 2 + 1); idx += 32) {
      const int g = idx / (N / 2 + 1), k = idx % (N / 2 + 1);
      if (k == 0) {
        const float a = RL.at(g, 0).x, b = RL.at(g, N).x;
        RL.at(g, 0) = make_float2(a + b, a - b);  // Ye = a + b, Yo = a - b (both real)
      } else {
        const float2 zk = RL.at(g, k), zn = RL.at(g, N - k);
        const float2 ye = cadd(zk, cconj(zn));
        const float2 yo = cmul(csub(zk, cconj(zn)), tw_pos(tw, k, m));
        if (k == N / 2) {
          RL.at(g, k) = make_float2(ye.x - yo.y, ye.y + yo.x);
        } else {
          const float2 ye2 = cadd(zn, cconj(zk));
          const float2 yo2 = cmul(csub(zn, cconj(zk)), tw_full<1>(tw, N - k, m));
          RL.at(g, k) = make_float2(ye.x - yo.y, ye.y + yo.x);
          RL.at(g, N - k) = make_float2(ye2.x - yo2.y, ye2.y + yo2.x);
        }
      }
    }
    __syncwarp();
    warp_fft<N, 1>(RL, G, tw);
    {  // p(2n) = Re z(n), p(2n+1) = Im z(n); keep v = (j - N/2) mod 2N
      float pv[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int idx = lane + 32 * t, g = idx / N, j = idx % N;
        const int v = (j - N / 2 + m) % m;
        const float2 zz = RL.at(g, v >> 1);
        pv[t] = ((v & 1) ? zz.y : zz.x) * scale_b;
      }
      __syncwarp();
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int idx = lane + 32 * t, g = idx / N, j = idx % N;
        RL.at(g, j).x = pv[t];
      }
    }
  }
  __syncthreads();
  // forward FFT of the real rows, two rows per complex line
  for (int r0 = warp * RP; r0 < N; r0 += kSmemWarps * RP) {
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int idx = lane + 32 * t, q = idx / N, j = idx % N;
      Z(r0 + 2 * q, j).y = Z(r0 + 2 * q + 1, j).x;
    }
    __syncwarp();
    warp_fft<N, -1>(PairLines<N>{Z, r0}, G, tw);
    pair_split<N>(Z, r0, lane);
  }
  __syncthreads();

  // ---- pass C: forward column FFT over kx in [0, N/2]
  for (int c0 = warp * G; c0 < HC; c0 += kSmemWarps * G)
    warp_fft<N, -1>(ColLines<N>{Z, c0}, min(G, HC - c0), tw);
  __syncthreads();
  // radial |F| sums in float32 (the reference sums in float32 with
  // scatter_add_): per lane, then a fixed xor tree across the warp. The bin
  // list holds plane offsets, the top bit set for columns 0 and N/2 (weight
  // 1; every other column stands for itself and its mirror, weight 2).
  for (int b = warp; b < P.n_bins; b += kSmemWarps) {
    float acc = 0.f;
    const int e1 = s_bptr[b + 1];
#pragma unroll 4
    for (int e = s_bptr[b] + lane; e < e1; e += 32) {
      const unsigned v = s_bins[e];
      const float2 f = Zs[v & 0x7fffu];
      const float a = sqrt_approx(fmaf(f.x, f.x, f.y * f.y));
      acc += (v & 0x8000u) ? a : 2.0f * a;
    }
    acc = warp_sum(acc);
    if (lane == 0) s_div[b] = (b == 0) ? 1.0f : __fdiv_rn(__ldg(P.bin_count + b), acc);
  }
  __syncthreads();

  // ---- pass D: radial divisor, inverse column FFT. The DC term (bin 0,
  // left as it is) over N^2 is the image mean; it is read before column 0
  // is transformed and taken out of every pixel in pass E, so the float32
  // plane-fit and variance sums run on centred values.
  if (threadIdx.x == 0) s_misc[0] = Z(0, 0).x * (float)(1.0 / ((double)N * (double)N));
  for (int c0 = warp * G; c0 < HC; c0 += kSmemWarps * G) {
    const int nc = min(G, HC - c0);
    for (int idx = lane; idx < nc * N; idx += 32) {
      const int cl = idx / N, r = idx % N, kx = c0 + cl;
      const int ky = r < N / 2 ? r : r - N;
      const int bin = (int)rintf(sqrt_approx((float)(ky * ky + kx * kx)));
      Z(r, kx) = cscale(Z(r, kx), s_div[bin]);
    }
    __syncwarp();
    warp_fft<N, 1>(ColLines<N>{Z, c0}, nc, tw);
  }
  __syncthreads();

  // ---- pass E: inverse row transform (real part) of row pairs, plane-fit
  // sums. Line q carries z = A + i B over the Hermitian extensions of rows
  // a = r0 + 2q and b = a + 1 (the imaginary parts of columns 0 and N/2 are
  // dropped, as the real part of the reference's ifft2 does); its inverse
  // is a + i b. Position N-k is written only from position k < N/2, which
  // no other task reads, so the packing needs no barrier.
  const float scale_e = (float)(1.0 / ((double)N * (double)N));
  const float mu = s_misc[0];
  float fz = 0.f, fxz = 0.f, fyz = 0.f, fww = 0.f;
  for (int r0 = warp * RP; r0 < N; r0 += kSmemWarps * RP) {
    for (int idx = lane; idx < G * HC; idx += 32) {
      const int q = idx / HC, k = idx - q * HC, i1 = r0 + 2 * q;
      const float2 a = Z(i1, k), b = Z(i1 + 1, k);
      if (k == 0 || k == N / 2) {
        Z(i1, k) = make_float2(a.x, b.x);
      } else {
        Z(i1, k) = make_float2(a.x - b.y, a.y + b.x);
        Z(i1, N - k) = make_float2(a.x + b.y, b.x - a.y);
      }
    }
    __syncwarp();
    warp_fft<N, 1>(PairLines<N>{Z, r0}, G, tw);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int idx = lane + 32 * t, q = idx / N, j = idx % N, i1 = r0 + 2 * q;
      const float2 z = Z(i1, j);
      const float wa = fmaf(z.x, scale_e, -mu), wb = fmaf(z.y, scale_e, -mu);
      Z(i1, j).x = wa;
      Z(i1 + 1, j).x = wb;
      fz += wa + wb;
      fxz = fmaf((float)i1, wa, fmaf((float)(i1 + 1), wb, fxz));
      fyz = fmaf((float)j, wa + wb, fyz);
      fww = fmaf(wa, wa, fmaf(wb, wb, fww));
    }
  }
  // Least-squares plane over the full N x N grid in closed form: the grid is
  // a Cartesian product, so the centred row and column coordinates are
  // orthogonal and the normal equations of the reference's 3x3 solve
  // (rows as x, columns as y) decouple.
  const float4 s4 = block_sum_f4<kSmemWarps>(make_float4(fz, fxz, fyz, fww), red4);
  constexpr float kMid = 0.5f * (float)(N - 1);
  constexpr float kSii = (float)((double)N * (double)N * ((double)N * (double)N - 1.0) / 12.0);
  const float pc0 = (s4.y - kMid * s4.x) / kSii;
  const float pc1 = (s4.z - kMid * s4.x) / kSii;
  const float pcm = s4.x * scale_e - (pc0 + pc1) * kMid;
  // Residual energy of the least-squares plane: sum (w - P)^2 = sum w^2 -
  // sum P w (the normal equations make the residual orthogonal to P). The
  // pixels are centred, so sum w^2 carries no DC term; where the plane
  // holds most of the energy the subtraction would cancel, and the residual
  // is summed directly instead (a block-uniform choice).
  float ssr = s4.w - fmaf(pc0, s4.y, fmaf(pc1, s4.z, pcm * s4.x));
  if (!(ssr > 0.25f * s4.w)) {
    float fsv = 0.f;
    for (int t = threadIdx.x; t < N * N; t += kSmemThreads) {
      const int i = t / N, j = t - i * N;
      const float v = Z(i, j).x - fmaf(pc0, (float)i, fmaf(pc1, (float)j, pcm));
      fsv = fmaf(v, v, fsv);
    }
    ssr = block_sum_f<kSmemWarps>(fsv, red);
  }
  const float sd = sqrtf(ssr * scale_e);
  const float inv_sd = sd > 1e-12f ? 1.0f / sd : 1.0f;

  // ---- pass F: normalise, mask, forward row FFT of row pairs
  for (int r0 = warp * RP; r0 < N; r0 += kSmemWarps * RP) {
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int idx = lane + 32 * t, q = idx / N, j = idx % N, i1 = r0 + 2 * q;
      const float pj = fmaf(pc1, (float)j, pcm);
      float fa = (Z(i1, j).x - fmaf(pc0, (float)i1, pj)) * inv_sd;
      float fb = (Z(i1 + 1, j).x - fmaf(pc0, (float)(i1 + 1), pj)) * inv_sd;
      if (P.mask != nullptr) {
        fa *= __ldg(P.mask + i1 * N + j);
        fb *= __ldg(P.mask + (i1 + 1) * N + j);
      }
      Z(i1, j) = make_float2(fa, fb);
    }
    __syncwarp();
    warp_fft<N, -1>(PairLines<N>{Z, r0}, G, tw);
    pair_split<N>(Z, r0, lane);
  }
  __syncthreads();
  // ---- pass G: forward column FFT
  for (int c0 = warp * G; c0 < HC; c0 += kSmemWarps * G)
    warp_fft<N, -1>(ColLines<N>{Z, c0}, min(G, HC - c0), tw);
  __syncthreads();
  // crop + pack + FSC, L2 norm (float32 per thread, fixed tree across the
  // block), pre-shifted write. Each thread keeps its packed values in
  // registers between the norm and the write, so once the norm's barrier is
  // passed the plane is free and the next template's plane load starts. The
  // packed index t = r * H + c advances by the block size with an add and
  // one carry, as H is a run-time size.
  constexpr int KP = (N * (N / 2 + 1) + kSmemThreads - 1) / kSmemThreads;
  const int dr = kSmemThreads / H, dc = kSmemThreads - dr * H;
  const int r_first = threadIdx.x / H, c_first = threadIdx.x - r_first * H;
  float2 fv[KP];
  float fss = 0.f;
  {
    int r = r_first, c = c_first;
#pragma unroll
    for (int q = 0; q < KP; ++q) {
      const int t = threadIdx.x + q * kSmemThreads;
      fv[q] = make_float2(0.f, 0.f);
      if (t < nb * H) {
        const int ky = r < nb / 2 ? r : r - nb;
        float2 f;
        if (c < nb / 2) f = Z((ky + N) & (N - 1), c);
        else if (nb == N) f = Z((ky + N) & (N - 1), N / 2);
        else f = cconj(Z((N - ky) & (N - 1), nb / 2));
        fv[q] = cscale(f, s_fsc[t]);
        fss = fmaf(fv[q].x, fv[q].x, fmaf(fv[q].y, fv[q].y, fss));
      }
      c += dc; r += dr;
      if (c >= H) { c -= H; ++r; }
    }
  }
  const float ss = block_sum_f<kSmemWarps>(fss, red);
  if (threadIdx.x == 0 && next_plane != nullptr) plane_load<N>(Zs, next_plane, bar);
  const float inv_norm = 1.0f / sqrtf(ss);
  float2* out = P.bank + (size_t)slot * nb * H;
  {
    int r = r_first, c = c_first;
#pragma unroll
    for (int q = 0; q < KP; ++q) {
      const int t = threadIdx.x + q * kSmemThreads;
      if (t < nb * H) {
        const int rs = r + nb / 2 < nb ? r + nb / 2 : r - nb / 2;
        const int cs = c + H / 2 < H ? c + H / 2 : c - (H - H / 2);
        out[(size_t)rs * H + cs] = cscale(fv[q], inv_norm);
      }
      c += dc; r += dr;
      if (c >= H) { c -= H; ++r; }
    }
  }
}

// Pass A as its own high-occupancy kernel: slice gather and pruned inverse
// along the 2N grid rows. A CTA takes kRiWarps * CPR columns of one
// template; a warp gathers its CPR columns into G = 2 * CPR staged lines
// (even and odd rows of the 2N grid), transforms them with one warp FFT and
// combines each even/odd pair into the N centred rows of the 2N-point
// inverse (output row (k + N/2) mod N takes frequency k). The CTA then
// writes its columns row by row into the template's plane in global memory,
// laid out as the shared-memory plane's rows (row stride plane_ld(N),
// column c at c + c/8), so the projector loads it with bulk copies. For box
// 256 the plane is the general kernel's unpadded [N][N+1] scratch layout,
// which that kernel's pass B reads directly.
constexpr int kRiWarps = 4;

template <int N>
__host__ __device__ constexpr bool flat_plane() { return N > 128; }
template <int N>
__host__ __device__ constexpr int plane_out_ld() { return flat_plane<N>() ? N + 1 : plane_ld(N); }

template <int N>
__host__ __device__ constexpr int ri_cols() { return kRiWarps * pass_a_cols<N>(); }

// Eight CTAs per SM (64 registers, 21 KB of shared memory): the gather is
// bound by the latency of its scattered loads, and resident warps hide it
// (measured on GB300 at box 128: 7 CTAs per SM 0.615 ms for the gather and
// tail of 768 templates, 8 CTAs 0.597 ms, 9 CTAs at 56 registers the same,
// 10 CTAs at 48 registers 0.644 ms; giving the L1 more of the SM's memory at
// the cost of resident CTAs was slower still). Streaming (evict-first) stores
// of the planes, to keep the blocked spectrum in L2, measured the same.
template <int N>
__global__ void __launch_bounds__(kRiWarps * 32, 8) rows_inverse(const float2* __restrict__ spectrum,
                                                              const float* __restrict__ rot,
                                                              const int* __restrict__ dirs,
                                                              const float2* __restrict__ tw_g,
                                                              float2* __restrict__ planes) {
  constexpr int m = 2 * N, W = N + 1, CPR = pass_a_cols<N>(), CC = ri_cols<N>(), LINE = plane_ld(N);
  constexpr int OUTC = CC + 1;
  static_assert(N * OUTC <= kRiWarps * 2 * CPR * LINE, "the output tile fits the staging lines");
  __shared__ float2 s_tw[kMaxFftLen / 2];
  // staging lines of the gather and the FFT; once every warp has its
  // outputs in registers, the same memory holds the CTA's N x CC output tile
  __shared__ float2 s_line[kRiWarps][2 * CPR][LINE];
  float2(*s_out)[OUTC] = reinterpret_cast<float2(*)[OUTC]>(&s_line[0][0][0]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y, c_cta = blockIdx.x * CC, cw = c_cta + warp * CPR;
  const int nc = max(0, min(CPR, W - cw));
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = tw_g[t];
  const float* R = rot + (size_t)dirs[b] * 9;
  float2(*L)[LINE] = s_line[warp];
  // Lanes take the warp's nc columns x 32/nc rows per load: samples of
  // neighbouring columns share trilinear corners. Against 32 rows of one
  // column this patch shape cut the gather's time by 40% on GB300; a
  // CTA-wide patch (8 columns x 4 rows per warp load) was slower again
  // (templates of a 64-candidate batch at box 128: 48.7 ms against 45.1).
  const int ncta = max(0, min(CC, W - c_cta));
#pragma unroll 4
  for (int idx = lane; idx < nc * m; idx += 32) {
    const int cl = idx % nc, r = idx / nc;
    const int k = r >> 1;
    L[2 * cl + (r & 1)][k + (k >> 3)] = slice_value<N>(spectrum, R, r, cw + cl);
  }
  __syncthreads();
  constexpr int RES = CPR * N / 32;  // outputs of a lane (8 at every box)
  float2 res[RES];
  if (nc > 0) {
    warp_fft<N, 1>(StageLines<N>{&L[0][0]}, 2 * nc, s_tw);
#pragma unroll
    for (int i = 0; i < RES; ++i) {
      const int idx = lane + 32 * i;
      if (idx < nc * N) {
        const int cl = idx / N, k = idx - cl * N;
        const int u = k < N / 2 ? k : k - N;
        const int kk = k + (k >> 3);
        res[i] = cadd(L[2 * cl][kk], cmul(tw_pos(s_tw, u, m), L[2 * cl + 1][kk]));
      }
    }
  }
  __syncthreads();  // every warp has read its lines
  if (nc > 0) {
#pragma unroll
    for (int i = 0; i < RES; ++i) {
      const int idx = lane + 32 * i;
      if (idx < nc * N) {
        const int cl = idx / N, k = idx - cl * N;
        s_out[(k + N / 2) & (N - 1)][warp * CPR + cl] = res[i];
      }
    }
  }
  __syncthreads();
  constexpr int OUT = plane_out_ld<N>();
  float2* dst = planes + (size_t)b * N * OUT;
  for (int e = threadIdx.x; e < N * CC; e += blockDim.x) {
    const int y = e / CC, cl = e - y * CC, c = c_cta + cl;
    if (cl < ncta) dst[(size_t)y * OUT + (flat_plane<N>() ? c : c + (c >> 3))] = s_out[y][cl];
  }
}

template <int N, int kSmemWarps>
__global__ void __launch_bounds__(32 * kSmemWarps, 1) project_templates_smem(ProjParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* Zs = reinterpret_cast<float2*>(smem_raw);
  float2* s_tw = Zs + plane_rows(N) * plane_ld(N);
  float4* red4 = reinterpret_cast<float4*>(s_tw + kMaxFftLen / 2);
  float* red = reinterpret_cast<float*>(red4 + kSmemMaxWarps);
  float* s_misc = red + kSmemMaxWarps;                                     // [4]
  uint64_t* bar = reinterpret_cast<uint64_t*>(s_misc + 4);
  float* s_div = reinterpret_cast<float*>(bar + 1);                         // [n_bins + 4]
  int* s_bptr = reinterpret_cast<int*>(s_div + P.n_bins + 4);              // [n_bins + 1]
  unsigned short* s_bins = reinterpret_cast<unsigned short*>(s_bptr + P.n_bins + 1);  // [N (N/2 + 1)]
  float* s_fsc = reinterpret_cast<float*>(s_bins + N * (N / 2 + 1));                  // [nb (nb/2 + 1)]
  constexpr int HC = N / 2 + 1;
  const Plane<N> Z{Zs};
  for (int t = threadIdx.x; t < P.nb * (P.nb / 2 + 1); t += blockDim.x) s_fsc[t] = P.fsc[t];
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = P.tw[t];
  for (int t = threadIdx.x; t <= P.n_bins; t += blockDim.x) s_bptr[t] = P.bin_ptr[t];
  // bin list as plane offsets (< 2^15 for N <= 128), top bit for the
  // columns that stand for themselves only
  for (int t = threadIdx.x; t < N * HC; t += blockDim.x) {
    const int idx = P.bin_list[t], r = idx / HC, kx = idx - r * HC;
    const unsigned edge = (kx == 0 || kx == N / 2) ? 0x8000u : 0u;
    s_bins[t] = (unsigned short)((unsigned)Z.off(r, kx) | edge);
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const size_t plane_elems = (size_t)N * plane_ld(N);
  if (threadIdx.x == 0 && blockIdx.x < P.n_build) plane_load<N>(Zs, P.planes + blockIdx.x * plane_elems, bar);
  uint32_t phase = 0;
  for (int b = blockIdx.x; b < P.n_build; b += gridDim.x, phase ^= 1u) {
    const int dir = P.dirs[b];
    const int slot = P.out_slot ? P.out_slot[b] : dir;
    const bool ok = plane_wait(bar, phase, P.wait_limit);
    if (__syncthreads_or(!ok)) {
      // a plane that did not arrive in time: the status word reports it;
      // the copy still in flight gets the default bound to land before the
      // CTA's shared memory is released; this template and the remaining
      // ones of the CTA become NaN, so every score computed from them is NaN
      if (threadIdx.x == 0) {
        if (P.status != nullptr) atomicExch(P.status, 1);
        plane_wait(bar, phase, kPlaneWaitLimit);
      }
      __syncthreads();
      const float nan = __int_as_float(0x7fc00000);
      for (int b2 = b; b2 < P.n_build; b2 += gridDim.x) {
        float2* out = P.bank + (size_t)(P.out_slot ? P.out_slot[b2] : P.dirs[b2]) * P.nb * (P.nb / 2 + 1);
        for (int t = threadIdx.x; t < P.nb * (P.nb / 2 + 1); t += blockDim.x) out[t] = make_float2(nan, nan);
      }
      return;
    }
    const int nxt = b + gridDim.x;
    build_one_smem<N, kSmemWarps>(P, slot, Zs, s_tw, s_div, red4, red, s_misc, s_bins, s_bptr, s_fsc,
                      nxt < P.n_build ? P.planes + nxt * plane_elems : nullptr, bar);
  }
}

}  // namespace

// complex elements of the blocked copy of one [2N][2N][N+1] spectrum
size_t project_blocked_elems(int N) { return (size_t)4 * N * N * ((N + 1 + kBX - 1) / kBX) * kBX; }

size_t project_smem_bytes_fast(int N, int n_bins, int nb) {
  return (size_t)plane_rows(N) * plane_ld(N) * sizeof(float2) + (kMaxFftLen / 2) * sizeof(float2) +
         kSmemMaxWarps * (sizeof(float4) + sizeof(float)) + 4 * sizeof(float) + sizeof(uint64_t) +
         (size_t)(n_bins + 4) * sizeof(float) + (size_t)(n_bins + 1) * sizeof(int) +
         (size_t)N * (N / 2 + 1) * sizeof(unsigned short) + (size_t)nb * (nb / 2 + 1) * sizeof(float);
}

template <int N, int NW>
static cudaError_t launch_tail(const ProjParams& P, int grid, size_t smem, cudaStream_t st) {
  static size_t set_smem = 0;  // attribute set once per size, never inside a stream capture
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(project_templates_smem<N, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  project_templates_smem<N, NW><<<grid, 32 * NW, smem, st>>>(P);
  return cudaGetLastError();
}

template <int N>
static cudaError_t launch_fast(ProjParams P, int grid, float2* planes, float2* blocked, cudaStream_t st) {
  constexpr int CC = ri_cols<N>();
  cudaError_t e0 = cudaSuccess;
  if (P.spectrum != nullptr) {  // else the blocked copy was written by the volume transform
    spectrum_blocked<N><<<8 * 152, 256, 0, st>>>(P.spectrum, blocked);
    e0 = cudaGetLastError();
    if (e0 != cudaSuccess) return e0;
  }
  rows_inverse<N><<<dim3((N + 1 + CC - 1) / CC, P.n_build), kRiWarps * 32, 0, st>>>(blocked, P.rot, P.dirs, P.tw,
                                                                                      planes);
  e0 = cudaGetLastError();
  if (e0 != cudaSuccess) return e0;
  P.planes = planes;
  const size_t smem = project_smem_bytes_fast(N, P.n_bins, P.nb);
  // 20 warps at box 128 (templates 4% faster than with 12 or 16, measured
  // on GB300 with 768 directions); 12 at the smaller boxes
  return launch_tail<N, N == 128 ? 20 : 12>(P, grid, smem, st);
}

cudaError_t launch_project_templates_fast(cudaStream_t st, const float2* spectrum, const float* rot,
                                          const int* dirs, int n_build, const int* out_slot,
                                          const float* mask, const float* fsc, const int* bin_list,
                                          const int* bin_ptr, const float* bin_count, int n_bins,
                                          const float2* tw, float2* bank, int grid, int N, int nb,
                                          float2* planes, float2* blocked, int* status, unsigned wait_limit) {
  if (n_build <= 0) return cudaSuccess;
  if (n_build > 65535) return cudaErrorInvalidValue;
  ProjParams P;
  P.status = status;
  P.wait_limit = wait_limit;
  P.spectrum = spectrum; P.rot = rot; P.dirs = dirs; P.n_build = n_build; P.mask = mask;
  P.fsc = fsc; P.bin_list = bin_list; P.bin_ptr = bin_ptr; P.bin_count = bin_count;
  P.n_bins = n_bins; P.tw = tw; P.tw3 = nullptr; P.bank = bank; P.out_slot = out_slot; P.scratch = nullptr;
  P.scratch_stride = 0; P.N = N; P.nb = nb; P.planes = nullptr;
  switch (N) {
    case 32: return launch_fast<32>(P, grid, planes, blocked, st);
    case 64: return launch_fast<64>(P, grid, planes, blocked, st);
    case 128: return launch_fast<128>(P, grid, planes, blocked, st);
    default: return cudaErrorInvalidValue;
  }
}

// Box 256: the slice gather and pass A run in rows_inverse from the blocked
// spectrum (its plane [N][N+1] written to global memory, ``chunk`` templates
// at a time), passes B-G in the general kernel, which reads those planes.
cudaError_t launch_project_templates_planes(cudaStream_t st, const float2* spectrum, const float* rot,
                                            const int* dirs, int n_build, const int* out_slot,
                                            const float* mask, const float* fsc, const int* bin_list,
                                            const int* bin_ptr, const float* bin_count, int n_bins,
                                            const float2* tw, const float2* tw3, float2* bank, float2* scratch,
                                            int grid, int N, int nb, float2* planes, float2* blocked, int chunk) {
  constexpr int kN = 256, CC = ri_cols<kN>();
  if (n_build <= 0) return cudaSuccess;
  if (N != kN || chunk <= 0 || chunk > 65535 || grid <= 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  if (spectrum != nullptr) {  // else the blocked copy was written by the volume transform
    spectrum_blocked<kN><<<8 * 152, 256, 0, st>>>(spectrum, blocked);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  ProjParams P;
  P.status = nullptr; P.wait_limit = 0;
  P.spectrum = spectrum; P.rot = rot; P.mask = mask; P.fsc = fsc; P.bin_list = bin_list; P.bin_ptr = bin_ptr;
  P.bin_count = bin_count; P.n_bins = n_bins; P.tw = tw; P.tw3 = tw3; P.bank = bank; P.scratch = scratch;
  P.scratch_stride = project_scratch_elems(N, nb); P.N = N; P.nb = nb; P.planes = planes;
  const size_t smem = project_smem_bytes(N, n_bins);
  for (int b0 = 0; b0 < n_build; b0 += chunk) {
    const int n = min(chunk, n_build - b0);
    rows_inverse<kN><<<dim3((kN + 1 + CC - 1) / CC, n), kRiWarps * 32, 0, st>>>(blocked, rot, dirs + b0, tw,
                                                                                 planes);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    P.dirs = dirs + b0; P.out_slot = out_slot ? out_slot + b0 : nullptr; P.n_build = n;
    e = launch_general<kN>(P, min(grid, n), smem, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// complex elements of the box-256 pass-A planes of ``n`` templates
size_t project_flat_plane_elems(int N, int n) { return (size_t)n * N * (N + 1); }
