// Correlation maximum over the translation window (v606:1418-1449) and the
// per-particle record statistics (v606:1466-1491), plain FP32, sm_103a.
//
// For a template T and a particle spectrum P (both stored pre-shifted, packed
// n x H, H = n/2+1), torch's irfft2 of Q = T * P on the crop window is
//     raw(y, x) = sum_{r,c} w_c Re[Q(r,c) exp(2 pi i (r y + c x)/n)]
// with w_c = 1 for c in {0, n/2} and 2 otherwise (the C2R keeps only the real
// part of those two columns); ccg = raw / n^2 and the score is 1024 * n^2 *
// max ccg = 1024 * max raw. Only y, x in [-C/2, C/2) are needed, so:
//   stage 1 (rows):  Z(y, c) = sum_q w_n^{q y} G_q(y mod 16, c), where
//                    G_q(., c) is a 16-point inverse DFT of Q(M j + q, c),
//                    j = 0..15, M = n/16, evaluated in registers;
//   stage 2 (cols):  raw(y, x) = sum_c Re[Z(y, c) w_c w_n^{c x}].
// One thread-block cluster per particle splits the H columns over its CTAs;
// each CTA keeps its columns of all psi spectra of the particle in shared
// memory (loaded with asynchronous copies), reads templates from L2, and the
// column partials of every map are summed over distributed shared memory by
// one CTA of the cluster (maps dealt out by rank), which takes the row-major
// first maximum. Per-map translation maps never reach HBM.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 256;
constexpr int kGroup = 5;     // templates per stage-1/stage-2 group (5 x 3 psi x 17 columns fills 256 threads at n = 128)
constexpr int kMaxLocal = 16; // templates whose partials are kept before a cluster reduction

struct CorrParams {
  const float2* bank;      // [n_templates][n][H]
  const float2* stack;     // [n_particles][n_psi][n][H]
  const int* local_ptr;    // [n_particles + 1]
  const int* local_idx;    // template index per entry
  const float2* tw_outer;  // [M][C]  exp(+2 pi i q y / n)
  const float2* tw_col;    // [H][C]  w_c exp(+2 pi i c x / n)
  float* out_score;        // [n_cand][nnz][n_psi]
  int* out_y;
  int* out_x;
  int n_particles, n_psi, n, cluster;
  int n_cand;              // candidates sharing the particle spectra
  long long bank_stride;   // complex elements between candidates' banks
  int nnz;                 // entries of the CSR (output stride per candidate)
  const unsigned char* subset;  // [n_cand][n_particles] nonzero: the candidate scores the particle (null: all)
};

// 8-byte asynchronous global-to-shared copy with an L2 evict-first hint:
// the particle spectra are read once per launch and should not push the
// templates out of L2.
__device__ __forceinline__ void cp_async8_stream(void* dst, const void* src, uint64_t policy) {
  asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src), "l"(policy)
               : "memory");
}

__host__ __device__ inline int col_lo(int H, int K, int r) {
  const int base = H / K, extra = H % K;
  return r * base + min(r, extra);
}

template <int C>
__global__ void __launch_bounds__(kThreads) correlate_plain(CorrParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int K = P.cluster;
  const int rank = (int)cluster.block_rank();
  const int b = blockIdx.x / K;
  const int n = P.n, H = n / 2 + 1, M = n / 16, n_psi = P.n_psi;
  const int clo = col_lo(H, K, rank), chi = col_lo(H, K, rank + 1), cw = chi - clo;
  const int cwmax = (H + K - 1) / K;
  constexpr int CC = C * C;
  constexpr int h = C / 2;

  float2* Pq = reinterpret_cast<float2*>(smem_raw);                 // [n_psi][n][cwmax]
  float2* Zb = Pq + (size_t)n_psi * n * cwmax;                       // [kGroup][n_psi][C][cwmax]
  float2* s_two = Zb + (size_t)kGroup * n_psi * C * cwmax;           // [M][C]
  float2* s_twc = s_two + (size_t)M * C;                             // [cwmax][C]
  float* rawp = reinterpret_cast<float*>(s_twc + (size_t)cwmax * C); // [kMaxLocal][n_psi][CC]

  const int e0 = P.local_ptr[b], d = P.local_ptr[b + 1] - e0;
  if (d <= 0) return;  // whole cluster returns together (same b)
  if (P.subset != nullptr) {  // a particle no candidate scores: nothing to do (same b for the cluster)
    bool any = false;
    for (int c = 0; c < P.n_cand && !any; ++c) any = P.subset[(size_t)c * P.n_particles + b] != 0;
    if (!any) return;
  }

  for (int t = threadIdx.x; t < M * C; t += blockDim.x) s_two[t] = P.tw_outer[t];
  for (int t = threadIdx.x; t < cw * C; t += blockDim.x) s_twc[t] = P.tw_col[(size_t)clo * C + t];
  // the particle's columns, all copies in flight at once (one wait)
  const float2* Pb = P.stack + (size_t)b * n_psi * n * H;
  {
    uint64_t policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
    for (int t = threadIdx.x; t < n_psi * n * cw; t += blockDim.x) {
      const int cl = t % cw, rr = t / cw;  // rr = psi * n + r
      cp_async8_stream(Pq + (size_t)rr * cwmax + cl, Pb + (size_t)rr * H + clo + cl, policy);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  }
  __syncthreads();

  for (int cand = 0; cand < P.n_cand; ++cand) {
  if (P.subset != nullptr && P.subset[(size_t)cand * P.n_particles + b] == 0) continue;  // cluster-uniform
  const float2* bank = P.bank + (size_t)cand * (size_t)P.bank_stride;
  const size_t out_base = (size_t)cand * P.nnz * n_psi;
  for (int sg = 0; sg < d; sg += kMaxLocal) {
    const int dsg = min(kMaxLocal, d - sg);
    for (int g0 = 0; g0 < dsg; g0 += kGroup) {
      const int gn = min(kGroup, dsg - g0);
      // ---- stage 1
      const int tasks = gn * n_psi * cw;
      for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
        const int cl = t % cw;
        const int gp = t / cw;
        const int psi = gp % n_psi, g = gp / n_psi;
        const int tmpl = P.local_idx[e0 + sg + g0 + g];
        const float2* T = bank + (size_t)tmpl * n * H + clo + cl;
        const float2* Pp = Pq + (size_t)psi * n * cwmax + cl;
        float2 Z[C];
#pragma unroll
        for (int yi = 0; yi < C; ++yi) Z[yi] = make_float2(0.f, 0.f);
        for (int q = 0; q < M; ++q) {
          float2 x[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int r = M * j + q;
            x[j] = cmul(__ldg(T + (size_t)r * H), Pp[(size_t)r * cwmax]);
          }
          idft16(x);
#pragma unroll
          for (int yi = 0; yi < C; ++yi) {
            const int rho = (yi - h) & 15;
            const float2 gq = x[idft16_slot(rho)];
            const float2 w = s_two[q * C + yi];
            Z[yi].x = fmaf(gq.x, w.x, fmaf(-gq.y, w.y, Z[yi].x));
            Z[yi].y = fmaf(gq.x, w.y, fmaf(gq.y, w.x, Z[yi].y));
          }
        }
        float2* zo = Zb + ((size_t)(g * n_psi + psi) * C) * cwmax + cl;
#pragma unroll
        for (int yi = 0; yi < C; ++yi) zo[(size_t)yi * cwmax] = Z[yi];
      }
      __syncthreads();
      // ---- stage 2: partial over this CTA's columns
      const int t2 = gn * n_psi * CC;
      for (int t = threadIdx.x; t < t2; t += blockDim.x) {
        const int xi = t % C;
        const int yi = (t / C) % C;
        const int gp = t / CC;  // g * n_psi + psi
        const float2* z = Zb + ((size_t)gp * C + yi) * cwmax;
        float acc = 0.f;
        for (int cl = 0; cl < cw; ++cl) {
          const float2 zz = z[cl], e = s_twc[cl * C + xi];
          acc = fmaf(zz.x, e.x, fmaf(-zz.y, e.y, acc));
        }
        rawp[((size_t)(g0 * n_psi) + gp) * CC + yi * C + xi] = acc;
      }
      __syncthreads();
    }
    // ---- cluster reduction and first-maximum search: the maps are dealt
    // out to the cluster's CTAs (map mp to rank mp mod K), each sums the K
    // partials of its maps over distributed shared memory in rank order
    cluster.sync();
    {
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      for (int mp = rank + K * warp; mp < dsg * n_psi; mp += K * nw) {
        float best = -INFINITY;
        int bi = CC;
        for (int e = lane; e < CC; e += 32) {
          float v = 0.f;
          for (int r = 0; r < K; ++r) {
            const float* rp = cluster.map_shared_rank(rawp, r);
            v += rp[(size_t)mp * CC + e];
          }
          if (v > best) { best = v; bi = e; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) {
          const int a = sg + mp / n_psi, psi = mp % n_psi;
          const size_t o = out_base + (size_t)(e0 + a) * n_psi + psi;
          P.out_score[o] = best * 1024.0f;
          P.out_y[o] = bi / C;
          P.out_x[o] = bi % C;
        }
      }
    }
    cluster.sync();
  }
  }
}

// One thread per particle: first maximum over (local direction, psi), the
// population mean and sigma of all its scores (FP64 sums in entry order),
// and the z-score. A particle has a few dozen scores at most, so a thread
// walks them itself (one warp per particle ran 32 times as many warps, most
// of their time in shuffle trees). A particle the candidate does not score
// (subset) gets the record of a particle without directions.
__global__ void particle_results(const int* __restrict__ local_ptr, const float* __restrict__ score,
                                 const int* __restrict__ ys, const int* __restrict__ xs, int n_particles,
                                 int n_psi, const unsigned char* __restrict__ subset, int* __restrict__ best_entry,
                                 int* __restrict__ best_psi, float* __restrict__ peak, int* __restrict__ peak_y,
                                 int* __restrict__ peak_x, float* __restrict__ zscore) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_particles) return;
  {  // candidate blockIdx.y: its scores follow the previous candidates'
    const int nnz = local_ptr[n_particles];
    const size_t so = (size_t)blockIdx.y * nnz * n_psi, po = (size_t)blockIdx.y * n_particles;
    score += so; ys += so; xs += so;
    best_entry += po; best_psi += po; peak += po; peak_y += po; peak_x += po; zscore += po;
  }
  const bool scored = subset == nullptr || subset[(size_t)blockIdx.y * n_particles + i] != 0;
  const int e0 = local_ptr[i], cnt = scored ? (local_ptr[i + 1] - e0) * n_psi : 0;
  if (cnt <= 0) {
    best_entry[i] = -1; best_psi[i] = -1; peak[i] = 0.f;
    peak_y[i] = 0; peak_x[i] = 0; zscore[i] = 0.f;
    return;
  }
  const float* s = score + (size_t)e0 * n_psi;
  float best = -INFINITY;
  int bi = 0;
  double sum = 0.0;
  for (int e = 0; e < cnt; ++e) {
    const float v = s[e];
    sum += (double)v;
    if (v > best) { best = v; bi = e; }
  }
  const double mean = sum / cnt;
  double var = 0.0;
  for (int e = 0; e < cnt; ++e) {
    const double dv = (double)s[e] - mean;
    var += dv * dv;
  }
  const double sd = sqrt(var / cnt);
  best_entry[i] = e0 + bi / n_psi;
  best_psi[i] = bi % n_psi;
  peak[i] = best;
  peak_y[i] = ys[(size_t)e0 * n_psi + bi];
  peak_x[i] = xs[(size_t)e0 * n_psi + bi];
  zscore[i] = (float)(((double)best - mean) / sd);
}

// sum over particles with at least one direction of exp(peak / 1024), FP64,
// fixed summation order. One cluster of kScoreCtas CTAs per candidate (on
// different SMs: GB300's FP64 rate is low, so one SM would spend tens of
// microseconds on the exponentials); CTA r sums a contiguous range of
// particles and rank 0 adds the partials in rank order.
constexpr int kScoreCtas = 8;

__global__ void __launch_bounds__(256) score_sum(const int* __restrict__ local_ptr, const float* __restrict__ peak,
                                                 int n_particles, const unsigned char* __restrict__ subset,
                                                 double* __restrict__ out) {
  __shared__ double red[32];
  __shared__ double part;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), cand = blockIdx.x / kScoreCtas;
  peak += (size_t)cand * n_particles;
  if (subset != nullptr) subset += (size_t)cand * n_particles;
  const int per = (n_particles + kScoreCtas - 1) / kScoreCtas;
  const int p0 = rank * per, p1 = min(n_particles, p0 + per);
  double acc = 0.0;
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x)
    if (local_ptr[p + 1] > local_ptr[p] && (subset == nullptr || subset[p] != 0))
      acc += exp((double)peak[p] / 1024.0);
  acc = block_sum_d(acc, red);
  if (threadIdx.x == 0) part = acc;
  cluster.sync();
  if (rank == 0 && threadIdx.x == 0) {
    double t = 0.0;
    for (int r = 0; r < kScoreCtas; ++r) t += *cluster.map_shared_rank(&part, r);
    out[cand] = t;
  }
  cluster.sync();
}

}  // namespace

int correlate_cluster_size(int n) {
  const int H = n / 2 + 1;
  int k = (H + 16) / 17;
  return k < 1 ? 1 : (k > 8 ? 8 : k);
}

// cluster: CTAs per particle (0: the default for n)
size_t correlate_smem_bytes(int n, int n_psi, int crop, int cluster) {
  const int H = n / 2 + 1, K = cluster > 0 ? cluster : correlate_cluster_size(n), cwmax = (H + K - 1) / K,
            M = n / 16;
  size_t b = (size_t)n_psi * n * cwmax * sizeof(float2);
  b += (size_t)kGroup * n_psi * crop * cwmax * sizeof(float2);
  b += (size_t)M * crop * sizeof(float2) + (size_t)cwmax * crop * sizeof(float2);
  b += (size_t)kMaxLocal * n_psi * crop * crop * sizeof(float);
  return b;
}

template <int C>
static cudaError_t launch_c(const CorrParams& P, size_t smem, cudaStream_t st) {
  static size_t set_smem = 0;  // attribute set once per size, never inside a stream capture
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(correlate_plain<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(P.n_particles * P.cluster));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)P.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, correlate_plain<C>, P);
}

cudaError_t launch_correlate_plain(cudaStream_t st, const float2* bank, const float2* stack,
                                   const int* local_ptr, const int* local_idx, int n_particles,
                                   int n_psi, int n, int crop, const float2* tw_outer,
                                   const float2* tw_col, float* out_score, int* out_y, int* out_x,
                                   int n_cand, long long bank_stride, int nnz, int cluster,
                                   const unsigned char* subset) {
  if (n_particles <= 0 || n_cand <= 0) return cudaSuccess;
  CorrParams P;
  P.n_cand = n_cand; P.bank_stride = bank_stride; P.nnz = nnz; P.subset = subset;
  P.bank = bank; P.stack = stack; P.local_ptr = local_ptr; P.local_idx = local_idx;
  P.tw_outer = tw_outer; P.tw_col = tw_col; P.out_score = out_score; P.out_y = out_y;
  P.out_x = out_x; P.n_particles = n_particles; P.n_psi = n_psi; P.n = n;
  P.cluster = cluster > 0 ? cluster : correlate_cluster_size(n);
  const size_t smem = correlate_smem_bytes(n, n_psi, crop, P.cluster);
  switch (crop) {
    case 2: return launch_c<2>(P, smem, st);
    case 4: return launch_c<4>(P, smem, st);
    case 6: return launch_c<6>(P, smem, st);
    case 8: return launch_c<8>(P, smem, st);
    case 10: return launch_c<10>(P, smem, st);
    case 12: return launch_c<12>(P, smem, st);
    case 14: return launch_c<14>(P, smem, st);
    case 16: return launch_c<16>(P, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_particle_results(cudaStream_t st, const int* local_ptr, const float* score,
                                    const int* ys, const int* xs, int n_particles, int n_psi,
                                    int* best_entry, int* best_psi, float* peak, int* peak_y,
                                    int* peak_x, float* zscore, int n_cand, const unsigned char* subset) {
  if (n_particles <= 0 || n_cand <= 0) return cudaSuccess;
  const int threads = 128;
  particle_results<<<dim3((n_particles + threads - 1) / threads, n_cand), threads, 0, st>>>(
      local_ptr, score, ys, xs, n_particles, n_psi, subset, best_entry, best_psi, peak, peak_y, peak_x, zscore);
  return cudaGetLastError();
}

cudaError_t launch_score_sum(cudaStream_t st, const int* local_ptr, const float* peak, int n_particles,
                             double* out, int n_cand, const unsigned char* subset) {
  if (n_cand <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n_cand * kScoreCtas));
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kScoreCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, score_sum, local_ptr, peak, n_particles, subset, out);
}
