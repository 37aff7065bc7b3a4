// Particle stack preparation (read_star_shift_crop_and_generate_new_star_v5.py).
//
// One batched pipeline per stack chunk, in float64 as the reference's numpy
// code computes it:
//   load       integer shift (zero fill) and centred crop into a complex
//              work array, one element per thread;
//   whiten     forward 2-D transform (cuFFT Z2Z, batched), then per image
//              the mean |F| of every radial bin (round(distance) on the
//              centred grid) and F *= 1 / mean (bin 0 keeps 1), inverse
//              transform (v5:42-59). The bins come as a CSR list of pixels
//              per bin, built once on the host; one CTA per image sums each
//              bin with a fixed lane order and a fixed shuffle tree, so the
//              result does not depend on scheduling;
//   normalize  least-squares plane over (column, row, value), subtracted,
//              then (v - mean) / population sigma when sigma > 0 (v5:61-106);
//              one CTA per image, fixed-order reductions;
//   highpass   forward transform, multiply by the raised-cosine edge mask
//              (a host table), inverse transform (v5:107-134);
//   store      the real part as float32.
// The transforms run in place on the work array; the 1/(h*w) of each
// inverse transform is applied where its output is next read.
#include "common.cuh"

namespace {

constexpr int kIngestThreads = 256;

__global__ void ingest_load(const float* __restrict__ images, int n, int h, int w, const int* __restrict__ shifts,
                            int ch, int cw, double2* __restrict__ work) {
  const long long total = (long long)n * ch * cw;
  const int y0 = h / 2 - ch / 2, x0 = w / 2 - cw / 2;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t % cw), r = (int)((t / cw) % ch);
    const long long img = t / ((long long)ch * cw);
    const int tx = shifts ? shifts[2 * img] : 0, ty = shifts ? shifts[2 * img + 1] : 0;
    // translated[y][x] = image[y - ty][x - tx] inside the image, else 0
    const int sy = y0 + r - ty, sx = x0 + c - tx;
    double v = 0.0;
    if (sy >= 0 && sy < h && sx >= 0 && sx < w) v = (double)images[(img * h + sy) * w + sx];
    work[t] = make_double2(v, 0.0);
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Per image: mean |F| per radial bin, then F *= 1 / mean (bin 0 and empty
// bins keep 1). Dynamic shared memory: n_bins doubles.
__global__ void __launch_bounds__(kIngestThreads) ingest_spectrum_divide(double2* __restrict__ work, int pixels,
                                                                         const int* __restrict__ bin_ptr,
                                                                         const int* __restrict__ bin_pix,
                                                                         const double* __restrict__ bin_count,
                                                                         int n_bins) {
  extern __shared__ double s_div[];
  double2* F = work + (size_t)blockIdx.x * pixels;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int b = warp; b < n_bins; b += nw) {
    double s = 0.0;
    for (int i = bin_ptr[b] + lane; i < bin_ptr[b + 1]; i += 32) {
      const double2 f = F[bin_pix[i]];
      s += hypot(f.x, f.y);
    }
    s = warp_sum_d(s);
    if (lane == 0) s_div[b] = (b == 0 || bin_count[b] <= 0.0) ? 1.0 : 1.0 / (s / bin_count[b]);
  }
  __syncthreads();
  for (int b = warp; b < n_bins; b += nw) {
    const double d = s_div[b];
    for (int i = bin_ptr[b] + lane; i < bin_ptr[b + 1]; i += 32) {
      double2 f = F[bin_pix[i]];
      f.x *= d;
      f.y *= d;
      F[bin_pix[i]] = f;
    }
  }
}

// Block-wide sum with a fixed tree (every thread gets the result).
__device__ double block_sum_d(double v, double* red) {
  v = warp_sum_d(v);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < nw; ++k) t += red[k];
  return t;
}

struct PlaneSums {
  double D, E, F, G, H, I;  // sums of x^2, xy, x, y^2, y, 1 over the pixel grid
};

// Plane fit, subtraction, mean and sigma normalisation of one image per CTA
// (v5:61-106). Input value = real part * scale. x = column, y = row.
__global__ void __launch_bounds__(kIngestThreads) ingest_normalize(double2* __restrict__ work, int ch, int cw,
                                                                   double scale, PlaneSums ps) {
  __shared__ double red[kIngestThreads / 32];
  const int pixels = ch * cw;
  double2* img = work + (size_t)blockIdx.x * pixels;
  double J = 0.0, K = 0.0, L = 0.0;
  for (int p = threadIdx.x; p < pixels; p += blockDim.x) {
    const double z = __dmul_rn(img[p].x, scale);
    const double x = (double)(p % cw), y = (double)(p / cw);
    J = __dadd_rn(J, __dmul_rn(x, z));
    K = __dadd_rn(K, __dmul_rn(y, z));
    L = __dadd_rn(L, z);
  }
  J = block_sum_d(J, red);
  K = block_sum_d(K, red);
  L = block_sum_d(L, red);
  const double D = ps.D, E = ps.E, F = ps.F, G = ps.G, H = ps.H, I = ps.I;
  const double denom = F * F * G - 2 * E * F * H + D * H * H + E * E * I - D * G * I;
  const double pa = (H * H * J - G * I * J + E * I * K + F * G * L - H * (F * K + E * L)) / denom;
  const double pb = (E * I * J + F * F * K - D * I * K + D * H * L - F * (H * J + E * L)) / denom;
  const double pc = (F * G * J - E * H * J - E * F * K + D * H * K + E * E * L - D * G * L) / denom;
  double s1 = 0.0, s2 = 0.0;
  for (int p = threadIdx.x; p < pixels; p += blockDim.x) {
    const double x = (double)(p % cw), y = (double)(p / cw);
    const double plane = __dadd_rn(__dadd_rn(__dmul_rn(pa, x), __dmul_rn(pb, y)), pc);
    const double v = __dsub_rn(__dmul_rn(img[p].x, scale), plane);
    img[p] = make_double2(v, 0.0);
    s1 = __dadd_rn(s1, v);
    s2 = __dadd_rn(s2, __dmul_rn(v, v));
  }
  s1 = block_sum_d(s1, red);
  s2 = block_sum_d(s2, red);
  const double n = (double)pixels;
  const double ave = s1 / n;
  const double sd = sqrt(__dsub_rn(s2 / n, __dmul_rn(ave, ave)));
  if (sd > 0.0) {
    for (int p = threadIdx.x; p < pixels; p += blockDim.x) img[p].x = (img[p].x - ave) / sd;
  }
}

// f *= scale (real part only, imaginary part cleared, when real_only), then
// f *= mask[pixel] when a mask is given.
__global__ void ingest_scale_mask(double2* __restrict__ work, long long total, int pixels,
                                  const double* __restrict__ mask, double scale, int real_only) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const double m = mask ? mask[t % pixels] : 1.0;
    double2 f = work[t];
    f.x = __dmul_rn(f.x, scale);
    f.y = real_only ? 0.0 : __dmul_rn(f.y, scale);
    if (mask) {
      f.x *= m;
      f.y *= m;
    }
    work[t] = f;
  }
}

__global__ void ingest_store(const double2* __restrict__ work, long long total, double scale,
                             float* __restrict__ out) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x)
    out[t] = (float)__dmul_rn(work[t].x, scale);
}

int grid_of(long long total, int sm_count) {
  long long g = (total + kIngestThreads - 1) / kIngestThreads;
  const long long cap = 8LL * sm_count;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

}  // namespace

cudaError_t launch_ingest_load(cudaStream_t st, const float* images, int n, int h, int w, const int* shifts, int ch,
                               int cw, double2* work, int sm_count) {
  ingest_load<<<grid_of((long long)n * ch * cw, sm_count), kIngestThreads, 0, st>>>(images, n, h, w, shifts, ch,
                                                                                   cw, work);
  return cudaGetLastError();
}

cudaError_t launch_ingest_spectrum_divide(cudaStream_t st, double2* work, int n, int pixels, const int* bin_ptr,
                                          const int* bin_pix, const double* bin_count, int n_bins) {
  const size_t smem = (size_t)n_bins * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(ingest_spectrum_divide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  ingest_spectrum_divide<<<n, kIngestThreads, smem, st>>>(work, pixels, bin_ptr, bin_pix, bin_count, n_bins);
  return cudaGetLastError();
}

cudaError_t launch_ingest_normalize(cudaStream_t st, double2* work, int n, int ch, int cw, double scale) {
  // sums over the pixel grid of x^2, xy, x, y^2, y and 1, exact in integers
  long long sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
  for (long long y = 0; y < ch; ++y)
    for (long long x = 0; x < cw; ++x) {
      sx += x; sy += y; sxx += x * x; syy += y * y; sxy += x * y;
    }
  PlaneSums ps{(double)sxx, (double)sxy, (double)sx, (double)syy, (double)sy, (double)((long long)ch * cw)};
  ingest_normalize<<<n, kIngestThreads, 0, st>>>(work, ch, cw, scale, ps);
  return cudaGetLastError();
}

cudaError_t launch_ingest_scale_mask(cudaStream_t st, double2* work, int n, int pixels, const double* mask,
                                     double scale, int real_only, int sm_count) {
  const long long total = (long long)n * pixels;
  ingest_scale_mask<<<grid_of(total, sm_count), kIngestThreads, 0, st>>>(work, total, pixels, mask, scale,
                                                                         real_only);
  return cudaGetLastError();
}

cudaError_t launch_ingest_store(cudaStream_t st, const double2* work, int n, int pixels, double scale, float* out,
                                int sm_count) {
  const long long total = (long long)n * pixels;
  ingest_store<<<grid_of(total, sm_count), kIngestThreads, 0, st>>>(work, total, scale, out);
  return cudaGetLastError();
}
