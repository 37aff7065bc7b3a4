// Shared device helpers for the GisAPR scoring kernels (sm_103a).
//
// Complex numbers are float2 (x = real, y = imaginary) in HBM and shared
// memory, matching torch.complex64 storage. Twiddle tables are computed on
// the host in double precision from the definition exp(-2*pi*i*k/L) and
// rounded once to float; no library trigonometry is reproduced here.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define GISAPR_DEV __device__ __forceinline__

// Largest 1-D transform length any kernel stages in shared memory.
constexpr int kMaxFftLen = 512;

GISAPR_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
GISAPR_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
GISAPR_DEV float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
GISAPR_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
GISAPR_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * conj(b) and conj(a) are folded into the twiddle sign by the callers.
GISAPR_DEV float2 cmul_sign(float2 a, float2 w, float sign) {
  // multiply by (w.x + i*sign*w.y)
  float wy = sign * w.y;
  return make_float2(a.x * w.x - a.y * wy, a.x * wy + a.y * w.x);
}

GISAPR_DEV int ilog2_pow2(int n) { return 31 - __clz(n); }
GISAPR_DEV int bitrev(int i, int logn) { return (int)(__brev((unsigned)i) >> (32 - logn)); }

// ---------------------------------------------------------------------------
// In-place radix-2 decimation-in-time FFT over many lines in shared memory.
//
// Line l, element k lives at buf[l * line_stride + k * elem_stride]. The data
// must already be in bit-reversed order along each line; the result is in
// natural order. sign = -1 for the forward transform exp(-2 pi i k n / L),
// +1 for the unnormalised inverse. ``tw`` holds exp(-2 pi i t / kMaxFftLen)
// for t < kMaxFftLen / 2. All threads of the block must call this.
// ---------------------------------------------------------------------------
GISAPR_DEV void smem_fft_dit(float2* buf, int L, int lines, int line_stride, int elem_stride,
                             float sign, const float2* __restrict__ tw) {
  // L, the butterfly span and the twiddle step are powers of two: the index
  // arithmetic is shifts and masks
  const int log_ht = ilog2_pow2(L) - 1, half_total = L >> 1;
  const int work = lines * half_total;
  constexpr int kLogMax = 9;  // log2(kMaxFftLen)
  static_assert((1 << kLogMax) == kMaxFftLen, "twiddle table length");
  for (int lh = 0, half = 1; half < L; ++lh, half <<= 1) {
    const int tw_shift = kLogMax - 1 - lh;  // twiddle step kMaxFftLen / (2 half)
    for (int t = threadIdx.x; t < work; t += blockDim.x) {
      const int line = t >> log_ht;
      const int b = t & (half_total - 1);
      const int k = b & (half - 1);
      const int i = ((b >> lh) << (lh + 1)) + k;
      float2* base = buf + line * line_stride;
      float2 u = base[i * elem_stride];
      float2 v = base[(i + half) * elem_stride];
      float2 w = tw[k << tw_shift];
      float2 vt = cmul_sign(v, w, -sign);  // tw is exp(-..): sign=-1 keeps it, +1 conjugates
      base[i * elem_stride] = cadd(u, vt);
      base[(i + half) * elem_stride] = csub(u, vt);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Transform lengths 3 * 2^k (boxes 96 and 192 and their doubled grids).
// ``tw3`` holds exp(-2 pi i t / kMaxFftLen3) for t < kMaxFftLen3 (the full
// circle), computed on the host like ``tw``.
// ---------------------------------------------------------------------------
constexpr int kMaxFftLen3 = 384;

GISAPR_DEV bool pow2_len(int L) { return (L & (L - 1)) == 0; }

// Position of input element j in the in-place layout smem_fft expects:
// bit-reversed for a power of two; for L = 3 L3, element 3q + r goes to
// sub-line r at the bit-reversed position of q.
GISAPR_DEV int fft_in_pos(int j, int L) {
  if (pow2_len(L)) return bitrev(j, ilog2_pow2(L));
  const int L3 = L / 3, q = j / 3, r = j - 3 * q;
  return r * L3 + bitrev(q, ilog2_pow2(L3));
}

// exp(+2 pi i num / den) for |num| <= den/2, den a power of two <= kMaxFftLen
// or 3 * 2^k <= kMaxFftLen3.
GISAPR_DEV float2 tw_pos_any(const float2* tw, const float2* tw3, int num, int den) {
  float2 w;
  if (pow2_len(den)) w = tw[abs(num) * (kMaxFftLen / den)];
  else w = tw3[abs(num) * (kMaxFftLen3 / den)];
  return num >= 0 ? make_float2(w.x, -w.y) : w;
}

// In-place transforms of ``lines`` contiguous lines of length L (line
// stride L) in shared memory, input in fft_in_pos order, output in natural
// order; sign -1 forward, +1 unnormalised inverse. For L = 3 L3 the three
// decimated sub-sequences are transformed by the radix-2 routine (as 3 x
// lines lines of L3) and combined by one radix-3 pass:
// X[k + m L3] = sum_r exp(sign 2 pi i r (k + m L3) / L) Y_r[k].
// All threads of the block must call this.
GISAPR_DEV void smem_fft(float2* buf, int L, int lines, float sign, const float2* __restrict__ tw,
                         const float2* __restrict__ tw3) {
  if (pow2_len(L)) {
    smem_fft_dit(buf, L, lines, L, 1, sign, tw);
    return;
  }
  const int L3 = L / 3, scale = kMaxFftLen3 / L;
  smem_fft_dit(buf, L3, 3 * lines, L3, 1, sign, tw);
  const float s3 = sign * 0.86602540378443864676f;  // Im exp(sign 2 pi i / 3)
  for (int t = threadIdx.x; t < lines * L3; t += blockDim.x) {
    const int l = t / L3, k = t - l * L3;
    float2* base = buf + (size_t)l * L;
    float2 w1 = tw3[k * scale], w2 = tw3[2 * k * scale];
    if (sign > 0.f) { w1.y = -w1.y; w2.y = -w2.y; }
    const float2 a = base[k], b = cmul(base[L3 + k], w1), c = cmul(base[2 * L3 + k], w2);
    const float2 s = cadd(b, c), d = csub(b, c);
    const float2 h = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
    base[k] = cadd(a, s);
    base[L3 + k] = make_float2(h.x - s3 * d.y, h.y + s3 * d.x);
    base[2 * L3 + k] = make_float2(h.x + s3 * d.y, h.y - s3 * d.x);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// 16-point inverse DFT in registers: X[r] = sum_j x[j] exp(+2 pi i j r / 16),
// as a radix-4 x radix-4 decomposition (j = 4 j1 + j2, r = r1 + 4 r2).
// The constants are cos/sin of multiples of pi/8.
// ---------------------------------------------------------------------------
GISAPR_DEV void idft4(float2& a, float2& b, float2& c, float2& d) {
  // X0 = a+b+c+d, X1 = a + i b - c - i d, X2 = a - b + c - d, X3 = a - i b - c + i d
  float2 s0 = cadd(a, c), s1 = csub(a, c), s2 = cadd(b, d), s3 = csub(b, d);
  float2 x0 = cadd(s0, s2);
  float2 x2 = csub(s0, s2);
  float2 ib = make_float2(-s3.y, s3.x);  // i * (b - d)
  float2 x1 = cadd(s1, ib);
  float2 x3 = csub(s1, ib);
  a = x0; b = x1; c = x2; d = x3;
}

GISAPR_DEV void idft16(float2 (&x)[16]) {
  constexpr float C1 = 0.92387953251128675613f;  // cos(pi/8)
  constexpr float S1 = 0.38268343236508977173f;  // sin(pi/8)
  constexpr float R2 = 0.70710678118654752440f;  // cos(pi/4)
  // Step 1: for each j2, a 4-point inverse DFT over j1 (elements j2, j2+4, ...).
#pragma unroll
  for (int j2 = 0; j2 < 4; ++j2) idft4(x[j2], x[j2 + 4], x[j2 + 8], x[j2 + 12]);
  // Now x[j2 + 4*r1] = A[j2][r1]. Twiddle by exp(+2 pi i j2 r1 / 16).
  // (j2, r1) products 1..9: angles k*pi/8.
  const float2 w1 = make_float2(C1, S1), w2 = make_float2(R2, R2), w3 = make_float2(S1, C1);
  const float2 w4 = make_float2(0.f, 1.f), w6 = make_float2(-R2, R2), w9 = make_float2(-C1, -S1);
  x[1 + 4] = cmul(x[1 + 4], w1);   // j2=1, r1=1
  x[1 + 8] = cmul(x[1 + 8], w2);   // j2=1, r1=2
  x[1 + 12] = cmul(x[1 + 12], w3); // j2=1, r1=3
  x[2 + 4] = cmul(x[2 + 4], w2);   // j2=2, r1=1
  x[2 + 8] = cmul(x[2 + 8], w4);   // j2=2, r1=2
  x[2 + 12] = cmul(x[2 + 12], w6); // j2=2, r1=3
  x[3 + 4] = cmul(x[3 + 4], w3);   // j2=3, r1=1
  x[3 + 8] = cmul(x[3 + 8], w6);   // j2=3, r1=2
  x[3 + 12] = cmul(x[3 + 12], w9); // j2=3, r1=3
  // Step 2: for each r1, a 4-point inverse DFT over j2: X[r1 + 4 r2].
#pragma unroll
  for (int r1 = 0; r1 < 4; ++r1)
    idft4(x[4 * r1 + 0], x[4 * r1 + 1], x[4 * r1 + 2], x[4 * r1 + 3]);
  // Now x[4*r1 + r2] holds X[r1 + 4*r2]; callers index through idft16_slot().
}

// Register slot that holds output r of idft16.
GISAPR_DEV constexpr int idft16_slot(int r) { return 4 * (r & 3) + (r >> 2); }

// ---------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------
GISAPR_DEV float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
GISAPR_DEV double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum of one double per thread (fixed tree order).
// ``scratch`` needs blockDim.x/32 doubles. Result is returned to every thread.
GISAPR_DEV double block_sum_d(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < nw ? scratch[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0) scratch[0] = t;
  }
  __syncthreads();
  t = scratch[0];
  __syncthreads();
  return t;
}

// Status word written by kernels that detect bad input on the device.
enum GisaprDeviceStatus : int {
  kDevOk = 0,
  kDevBadIndex = 1,
  kDevTooManyLocal = 2,
};

// ---------------------------------------------------------------------------
// Register DFT codelets, natural-order outputs.
// dft<R, DIR>: X[k] = sum_n x[n] exp(DIR * 2 pi i n k / R), DIR = -1 forward,
// +1 inverse (unnormalised). Constants are cos/sin of multiples of pi/8.
// ---------------------------------------------------------------------------
template <int DIR>
GISAPR_DEV float2 mul_dir_i(float2 a) {  // a * (DIR * i)
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int DIR>
GISAPR_DEV void dft2(float2& a, float2& b) {
  float2 s = cadd(a, b), d = csub(a, b);
  a = s; b = d;
}

template <int DIR>
GISAPR_DEV void dft4(float2& a, float2& b, float2& c, float2& d) {
  const float2 s0 = cadd(a, c), s1 = csub(a, c), s2 = cadd(b, d), s3 = csub(b, d);
  const float2 t = mul_dir_i<DIR>(s3);
  a = cadd(s0, s2);
  c = csub(s0, s2);
  b = cadd(s1, t);
  d = csub(s1, t);
}

// exp(DIR * i * k * pi / 8) for k = 0..15
template <int DIR>
GISAPR_DEV float2 w16(int k) {
  constexpr float C1 = 0.92387953251128675613f, S1 = 0.38268343236508977173f, R2 = 0.70710678118654752440f;
  float c, s;
  switch (k & 15) {
    case 0: c = 1.f; s = 0.f; break;
    case 1: c = C1; s = S1; break;
    case 2: c = R2; s = R2; break;
    case 3: c = S1; s = C1; break;
    case 4: c = 0.f; s = 1.f; break;
    case 5: c = -S1; s = C1; break;
    case 6: c = -R2; s = R2; break;
    case 7: c = -C1; s = S1; break;
    case 8: c = -1.f; s = 0.f; break;
    case 9: c = -C1; s = -S1; break;
    case 10: c = -R2; s = -R2; break;
    case 11: c = -S1; s = -C1; break;
    case 12: c = 0.f; s = -1.f; break;
    case 13: c = S1; s = -C1; break;
    case 14: c = R2; s = -R2; break;
    default: c = C1; s = -S1; break;
  }
  return make_float2(c, DIR > 0 ? s : -s);
}

template <int R, int DIR>
GISAPR_DEV void dft(float2 (&x)[R]);

template <>
GISAPR_DEV void dft<2, 1>(float2 (&x)[2]) { dft2<1>(x[0], x[1]); }
template <>
GISAPR_DEV void dft<2, -1>(float2 (&x)[2]) { dft2<-1>(x[0], x[1]); }

template <>
GISAPR_DEV void dft<4, 1>(float2 (&x)[4]) { dft4<1>(x[0], x[1], x[2], x[3]); }
template <>
GISAPR_DEV void dft<4, -1>(float2 (&x)[4]) { dft4<-1>(x[0], x[1], x[2], x[3]); }

// 8 = 2 x 4: n = 4 n1 + n2, k = k1 + 2 k2
template <int DIR>
GISAPR_DEV void dft8_impl(float2 (&x)[8]) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft2<DIR>(x[n2], x[n2 + 4]);  // x[n2 + 4 k1] = A[n2][k1]
  // twiddle A[n2][1] by exp(DIR 2 pi i n2 / 8) = w16(2 n2)
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2) x[n2 + 4] = cmul(x[n2 + 4], w16<DIR>(2 * n2));
  dft4<DIR>(x[0], x[1], x[2], x[3]);  // k1 = 0 -> X[0], X[2], X[4], X[6]
  dft4<DIR>(x[4], x[5], x[6], x[7]);  // k1 = 1 -> X[1], X[3], X[5], X[7]
  float2 y[8];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    y[2 * k2] = x[k2];
    y[2 * k2 + 1] = x[4 + k2];
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = y[k];
}
template <>
GISAPR_DEV void dft<8, 1>(float2 (&x)[8]) { dft8_impl<1>(x); }
template <>
GISAPR_DEV void dft<8, -1>(float2 (&x)[8]) { dft8_impl<-1>(x); }

// 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2
template <int DIR>
GISAPR_DEV void dft16_impl(float2 (&x)[16]) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4<DIR>(x[n2], x[n2 + 4], x[n2 + 8], x[n2 + 12]);
  // x[n2 + 4 k1] = A[n2][k1]; twiddle by exp(DIR 2 pi i n2 k1 / 16) = w16(n2 k1)
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) x[n2 + 4 * k1] = cmul(x[n2 + 4 * k1], w16<DIR>(n2 * k1));
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(x[4 * k1 + 0], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
  // x[4 k1 + k2] = X[k1 + 4 k2]
  float2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) y[k1 + 4 * k2] = x[4 * k1 + k2];
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = y[k];
}
template <>
GISAPR_DEV void dft<16, 1>(float2 (&x)[16]) { dft16_impl<1>(x); }
template <>
GISAPR_DEV void dft<16, -1>(float2 (&x)[16]) { dft16_impl<-1>(x); }

// exp(DIR * 2 pi i * t / L) from the half table tw[t'] = exp(-2 pi i t' / kMaxFftLen),
// t' < kMaxFftLen / 2, for any integer t (L divides kMaxFftLen).
template <int DIR>
GISAPR_DEV float2 tw_full(const float2* __restrict__ tw, int t, int L) {
  int u = (t * (kMaxFftLen / L)) & (kMaxFftLen - 1);
  float2 w = u < kMaxFftLen / 2 ? tw[u] : make_float2(-tw[u - kMaxFftLen / 2].x, -tw[u - kMaxFftLen / 2].y);
  return DIR < 0 ? w : make_float2(w.x, -w.y);
}

// ---------------------------------------------------------------------------
// The reference's real-space gridding correction (v606:837-853): the padded
// volume is multiplied by sinc(|f|)^2, f the fftshifted fftfreq of the 2N grid.
// ---------------------------------------------------------------------------
GISAPR_DEV float fftfreq_shifted_f32(int i, int m) {
  // fftshift(fftfreq(m))[i] = (i - m/2) * float(1/m)
  return __fmul_rn((float)(i - m / 2), (float)(1.0 / (double)m));
}

// float32 sinc(r)^2 in the operation order of the reference filter
// (v606:841-853 with torch.sinc: sin(pi*r)/(pi*r), 1 at r == 0).
GISAPR_DEV float sinc2_f32(float fz2, float fy2, float fx2) {
  float r = sqrtf(__fadd_rn(__fadd_rn(fz2, fy2), fx2));
  float s;
  if (r == 0.0f) {
    s = 1.0f;
  } else {
    float prod = __fmul_rn(3.14159274101257324219f, r);
    s = __fdiv_rn(sinf(prod), prod);
  }
  return __fmul_rn(s, s);
}

