// Packed CTF*ISSPA table and particle spectra (v606:695-829, 1193-1374).
//
// packed_ctf: one thread per packed coefficient of one particle. The static
// frequency terms (x, y, u^4, ISSPA noise curve) are host tables built with
// the reference's float32 numpy expressions; the per-particle trigonometry
// and the phase gamma repeat the reference's float32 operation order without
// fused multiply-add, because gamma reaches hundreds of radians and a single
// rounding difference moves sin(gamma) by ~1e-5.
//
// prepare_particles: one CTA per (particle, psi). Rows of the rotated image
// (bilinear, zero padding, align_corners=True, in the weight order of
// torch's vectorised 2-D CPU kernel) are masked and transformed in shared
// memory, then columns; the packed half plane is Fourier-cropped, multiplied
// by the CTF table, conjugated, L2-normalised and written pre-shifted.
#include "common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kRowBatch = 8;
constexpr int kColBatch = 16;

struct CtfConst {
  float k1, k2, k3, k5, kk;
};

__global__ void packed_ctf(const float* __restrict__ dfu, const float* __restrict__ dfv,
                           const float* __restrict__ dfa, int n, const float* __restrict__ tx,
                           const float* __restrict__ ty, const float* __restrict__ tu4,
                           const float* __restrict__ tnc, int K, CtfConst c,
                           float* __restrict__ out) {
  const int p = blockIdx.y;
  if (p >= n) return;
  // angle = deg2rad(dfa) in float32: dfa * float(pi/180)
  const float ang = __fmul_rn(dfa[p], (float)(3.14159265358979323846 / 180.0));
  const float sa = sinf(ang), ca = cosf(ang);
  const float u = dfu[p], v = dfv[p];
  const float axx = __fsub_rn(__fmul_rn(__fmul_rn(-u, ca), ca), __fmul_rn(__fmul_rn(v, sa), sa));
  const float ayy = __fsub_rn(__fmul_rn(__fmul_rn(-u, sa), sa), __fmul_rn(__fmul_rn(v, ca), ca));
  const float axy = __fadd_rn(__fmul_rn(__fmul_rn(-u, sa), ca), __fmul_rn(__fmul_rn(v, sa), ca));
  const float axy2 = __fmul_rn(2.0f, axy);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const float x = tx[k], y = ty[k];
    const float t1 = __fmul_rn(__fmul_rn(axx, x), x);
    const float t2 = __fmul_rn(__fmul_rn(axy2, x), y);
    const float t3 = __fmul_rn(__fmul_rn(ayy, y), y);
    const float s = __fadd_rn(__fadd_rn(t1, t2), t3);
    float g = __fmul_rn(c.k1, s);
    g = __fadd_rn(g, __fmul_rn(c.k2, tu4[k]));
    g = __fsub_rn(g, c.k5);
    g = __fsub_rn(g, c.k3);
    float val = -sinf(g);
    if (fabsf(val) < 1e-8f) val = (val > 0.f) ? 1e-8f : ((val < 0.f) ? -1e-8f : 0.f);
    const float den = __fadd_rn(tnc[k], __fmul_rn(__fmul_rn(c.kk, val), val));
    const float w = __fmul_rn(val, sqrtf(__frcp_rn(den)));
    out[(size_t)p * K + k] = w;
  }
}

struct PrepParams {
  const float* images;     // [n][N][N]
  const int* psi_index;    // [n][n_psi] index into psi table
  const float4* psi_tab;   // (cos, sin, off_row, off_col) float32 per psi angle
  const float* mask;       // [N][N] or null
  const float* ctf;        // [n][nb][H]
  float2* out;             // [n][n_psi][nb][H]
  float2* scratch;
  size_t scratch_stride;
  const float2* tw;
  const float2* tw3;       // twiddles of lengths 3 * 2^k
  int n, n_psi, N, nb;
};

__device__ __forceinline__ float sample_bilinear_zero(const float* __restrict__ img, int N,
                                                      float iy, float ix) {
  const float fy = floorf(iy), fx = floorf(ix);
  const int y0 = (int)fy, x0 = (int)fx;
  const float w = __fsub_rn(ix, fx), e = __fsub_rn(1.0f, w);
  const float nn = __fsub_rn(iy, fy), s = __fsub_rn(1.0f, nn);
  const float wnw = __fmul_rn(s, e), wne = __fmul_rn(s, w);
  const float wsw = __fmul_rn(nn, e), wse = __fmul_rn(nn, w);
  auto at = [&](int yy, int xx) -> float {
    return (yy >= 0 && yy < N && xx >= 0 && xx < N) ? __ldg(img + (size_t)yy * N + xx) : 0.0f;
  };
  float acc = __fmul_rn(at(y0, x0), wnw);
  acc = __fadd_rn(acc, __fmul_rn(at(y0, x0 + 1), wne));
  acc = __fadd_rn(acc, __fmul_rn(at(y0 + 1, x0), wsw));
  acc = __fadd_rn(acc, __fmul_rn(at(y0 + 1, x0 + 1), wse));
  return acc;
}

__global__ void __launch_bounds__(kThreads) prepare_particles(PrepParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = P.N, nb = P.nb, H = nb / 2 + 1, HC = N / 2 + 1;
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  float2* s_tw = sm + max(kRowBatch, kColBatch) * N;
  double* red = reinterpret_cast<double*>(s_tw + kMaxFftLen / 2);
  for (int t = threadIdx.x; t < kMaxFftLen / 2; t += blockDim.x) s_tw[t] = P.tw[t];
  __syncthreads();
  float2* S = P.scratch + (size_t)blockIdx.x * P.scratch_stride;
  float2* Pk = S + (size_t)N * HC;
  const float half = __fdiv_rn((float)(N - 1), 2.0f);
  const float nm1 = (float)(N - 1);
  for (int job = blockIdx.x; job < P.n * P.n_psi; job += gridDim.x) {
    const int p = job / P.n_psi, si = job - p * P.n_psi;
    const float4 ps = P.psi_tab[P.psi_index[(size_t)p * P.n_psi + si]];
    const float cth = ps.x, sth = ps.y;
    const float* img = P.images + (size_t)p * N * N;
    // rows: rotate, mask, forward FFT
    for (int i0 = 0; i0 < N; i0 += kRowBatch) {
      const int nr = min(kRowBatch, N - i0);
      for (int t = threadIdx.x; t < nr * N; t += blockDim.x) {
        const int rl = t / N, j = t - rl * N;
        const float yy = (float)(i0 + rl), xx = (float)j;
        // source = [row, col] @ M^T + offset; M = [[c, -s], [s, c]]
        const float sy = __fadd_rn(__fmaf_rn(-sth, xx, __fmul_rn(cth, yy)), ps.z);
        const float sx = __fadd_rn(__fmaf_rn(cth, xx, __fmul_rn(sth, yy)), ps.w);
        const float yn = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, sy), nm1), 1.0f);
        const float xn = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, sx), nm1), 1.0f);
        const float iy = __fmul_rn(__fadd_rn(yn, 1.0f), half);
        const float ix = __fmul_rn(__fadd_rn(xn, 1.0f), half);
        float v = sample_bilinear_zero(img, N, iy, ix);
        if (P.mask != nullptr) v = __fmul_rn(v, P.mask[(size_t)(i0 + rl) * N + j]);
        sm[rl * N + fft_in_pos(j, N)] = make_float2(v, 0.f);
      }
      __syncthreads();
      smem_fft(sm, N, nr, -1.0f, s_tw, P.tw3);
      for (int t = threadIdx.x; t < nr * HC; t += blockDim.x) {
        const int rl = t / HC, k = t - rl * HC;
        S[(size_t)(i0 + rl) * HC + k] = sm[rl * N + k];
      }
      __syncthreads();
    }
    // columns
    for (int c0 = 0; c0 < HC; c0 += kColBatch) {
      const int nc = min(kColBatch, HC - c0);
      for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
        const int r = t / nc, cl = t - r * nc;
        sm[cl * N + fft_in_pos(r, N)] = S[(size_t)r * HC + c0 + cl];
      }
      __syncthreads();
      smem_fft(sm, N, nc, -1.0f, s_tw, P.tw3);
      for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
        const int r = t / nc, cl = t - r * nc;
        S[(size_t)r * HC + c0 + cl] = sm[cl * N + r];
      }
      __syncthreads();
    }
    // crop, pack, CTF, conjugate, norm
    const float* ctf = P.ctf + (size_t)p * nb * H;
    double ss = 0.0;
    for (int t = threadIdx.x; t < nb * H; t += blockDim.x) {
      const int r = t / H, c = t - r * H;
      const int ky = r < nb / 2 ? r : r - nb;
      float2 f;
      if (c < nb / 2) f = S[(size_t)((ky + N) % N) * HC + c];
      else if (nb == N) f = S[(size_t)((ky + N) % N) * HC + N / 2];
      else f = cconj(S[(size_t)((-ky + N) % N) * HC + nb / 2]);
      const float w = ctf[t];
      f = make_float2(__fmul_rn(f.x, w), -__fmul_rn(f.y, w));
      Pk[t] = f;
      ss += (double)f.x * f.x + (double)f.y * f.y;
    }
    ss = block_sum_d(ss, red);
    const float inv = (float)(1.0 / sqrt(ss));
    float2* out = P.out + ((size_t)p * P.n_psi + si) * nb * H;
    for (int t = threadIdx.x; t < nb * H; t += blockDim.x) {
      const int r = t / H, c = t - r * H;
      const int rs = (r + nb / 2) % nb, cs = (c + H / 2) % H;
      out[(size_t)rs * H + cs] = cscale(Pk[t], inv);
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_packed_ctf(cudaStream_t st, const float* dfu, const float* dfv, const float* dfa,
                              int n, const float* tx, const float* ty, const float* tu4,
                              const float* tnc, int K, float k1, float k2, float k3, float k5,
                              float kk, float* out) {
  if (n <= 0) return cudaSuccess;
  CtfConst c{k1, k2, k3, k5, kk};
  dim3 grid((K + 255) / 256, n);
  packed_ctf<<<grid, 256, 0, st>>>(dfu, dfv, dfa, n, tx, ty, tu4, tnc, K, c, out);
  return cudaGetLastError();
}

size_t prepare_scratch_elems(int N, int nb) {
  return (size_t)N * (N / 2 + 1) + (size_t)nb * (nb / 2 + 1);
}

size_t prepare_smem_bytes(int N) {
  return (size_t)max(kRowBatch, kColBatch) * N * sizeof(float2) + (kMaxFftLen / 2) * sizeof(float2) +
         40 * sizeof(double);
}

cudaError_t launch_prepare_particles(cudaStream_t st, const float* images, int n, int n_psi,
                                     const int* psi_index, const void* psi_tab, const float* mask,
                                     const float* ctf, float2* out, float2* scratch, int grid,
                                     const float2* tw, const float2* tw3, int N, int nb) {
  if (n <= 0) return cudaSuccess;
  PrepParams P;
  P.images = images; P.psi_index = psi_index; P.psi_tab = (const float4*)psi_tab; P.mask = mask;
  P.ctf = ctf; P.out = out; P.scratch = scratch; P.scratch_stride = prepare_scratch_elems(N, nb);
  P.tw = tw; P.tw3 = tw3; P.n = n; P.n_psi = n_psi; P.N = N; P.nb = nb;
  const size_t smem = prepare_smem_bytes(N);
  static size_t set_smem = 0;
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(prepare_particles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  prepare_particles<<<grid, kThreads, smem, st>>>(P);
  return cudaGetLastError();
}
