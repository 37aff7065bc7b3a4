// Tensor-core correlation for batches of candidates (tcgen05, TMEM), sm_103a.
//
// The crop-window transform of the plain kernel is, per packed column c,
//     Z_{m,s}(y, c) = sum_r T_m(r, c) * P_s(r, c) * w_n^{r y}          (stage 1)
//     raw_{m,s}(y, x) = sum_c Re[Z_{m,s}(y, c) w_c w_n^{c x}]         (stage 2)
// for rows m = (local direction, candidate) of one particle and its psi
// angles s. For a fixed particle and column, stage 1 is a complex GEMM
// between the rows' template columns T_m(., c) and U_{s,y}(r) = P_s(r,c) w^{ry},
// shared by every candidate: in real form D[m][j] = sum_k A[m][k] B[j][k] with
// A = [Re T | Im T] (K = 2n) and B's row j = (s, y, part) holding
// [Re U | -Im U] (part 0, Re Z) or [Im U | Re U] (part 1, Im Z).
//
// Precision: both operands are scaled by 2^13 (every entry has modulus <= 1,
// the packed spectra having unit L2 norm) and split into fp16 hi + lo parts;
// the split form accumulates hi*hi + hi*lo + lo*hi in FP32 (three passes of
// tcgen05.mma over K), which keeps about 22 significant bits per product.
// The single form uses hi*hi only.
//
// One CTA takes one particle, a tile of 128 rows (row = a * n_cand + cand,
// so a tile holds whole directions and the work list, sorted by direction,
// lets concurrent CTAs share template columns in L2) and a group of up to
// three psi angles. For each column it
// copies the rows' template columns (fp16 hi/lo, column-major copy of the
// banks) with cp.async, builds B in shared memory, and one thread issues the
// MMAs (M=128, N=kN, K=16, FP32 accumulate into one of two TMEM buffers) and
// commits to an mbarrier. While the tensor cores run column c, twelve warps
// read column c-1 from the other TMEM buffer (tcgen05.ld) and accumulate
// stage 2 on CUDA cores in registers; after the last column each thread takes
// the row-major first maximum of its (row, psi) map. Operands use the
// canonical K-major no-swizzle layout: 8x8 fp16 core matrices of 128
// contiguous bytes, LBO = 128 B along K, SBO = (K/8)*128 B between 8-row
// groups. Every mbarrier wait is bounded; on timeout the kernel sets *status,
// waits (bounded) for the MMA in flight, frees TMEM and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kTcThreads = 384;   // 12 warps: 3 per TMEM lane quarter
constexpr int kTcM = 128;         // rows per tile (TMEM lanes)
constexpr int kTcPsi = 3;         // psi angles per particle held by a tile
constexpr int kTcMaxN = 128;      // K = 2n <= 256 staged in one pass
constexpr int kTcTmemCols = 256;  // two accumulator buffers of kN <= 80 columns
constexpr float kTcScale = 8192.0f;               // 2^13 on each operand
constexpr float kTcUnscale = 1.0f / 67108864.0f;  // 2^-26 for the product
constexpr unsigned kWaitLimit = 1u << 24;         // bounded mbarrier spin

// TMEM / B-row stride of one psi angle: crop x (re, im), rounded up to 8 so
// every tcgen05.ld starts on an 8-column boundary.
__host__ __device__ constexpr int tc_psi_stride(int C) { return ((2 * C + 7) / 8) * 8; }
// MMA N: all psi angles, rounded up to a multiple of 16.
__host__ __device__ constexpr int tc_n(int C) { return ((kTcPsi * tc_psi_stride(C) + 15) / 16) * 16; }

struct TcParams {
  const __half* tbank;    // [n_cand][n_slot][H][2][K]: hi then lo of [Re T(r) | Im T(r)], scaled
  long long cand_stride;  // halves between candidates
  const float2* stack;    // [n_particles][n_psi][n][H]
  const int* local_ptr;
  const int* local_idx;
  const int* work;        // [n_work][2]: particle, tile * n_groups + psi group
  int n_work, n_cand, n_psi, n, nnz, split;
  const float2* tw_row;   // [n]  exp(+2 pi i t / n)
  const float2* tw_col;   // [H][C]  w_c exp(+2 pi i c (x - h) / n)
  float* out_score;       // [n_cand][nnz][n_psi]
  int* out_y;
  int* out_x;
  int* status;            // set to 1 when an mbarrier wait ran out
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, no swizzle (K-major core matrices).
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, relative LBO, no swizzle
}

// kind::f16 instruction descriptor: FP32 accumulate, F16 A and B, both K-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row, k) in a K-major tile with K columns
__device__ __forceinline__ uint32_t core_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// Wait for the barrier phase of the given parity with an iteration limit;
// returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity));
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src));
}

__device__ __forceinline__ void st_half2(unsigned char* p, __half2 v) {
  *reinterpret_cast<__half2*>(p) = v;
}

// hi = fp16(a, b); lo = fp16(a - hi, b - hi)
__device__ __forceinline__ void split2(float a, float b, __half2& hi, __half2& lo) {
  hi = __floats2half2_rn(a, b);
  const float2 hf = __half22float2(hi);
  lo = __floats2half2_rn(a - hf.x, b - hf.y);
}

// Accumulate stage 2 for NY crop rows starting at yi0 from a TMEM load of
// 2 * NY columns (re, im per row).
template <int C, int NY>
__device__ __forceinline__ void stage2_rows(float (&acc)[C][C], const uint32_t (&v)[8], int yi0,
                                            const float2* __restrict__ twc) {
#pragma unroll
  for (int xi = 0; xi < C; ++xi) {
    const float2 e = twc[xi];
#pragma unroll
    for (int yy = 0; yy < NY; ++yy) {
      const float zr = __uint_as_float(v[2 * yy]), zi = __uint_as_float(v[2 * yy + 1]);
      acc[yi0 + yy][xi] = fmaf(zr, e.x, fmaf(-zi, e.y, acc[yi0 + yy][xi]));
    }
  }
}

template <int C>
__global__ void __launch_bounds__(kTcThreads, 1) correlate_tc(TcParams P) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr int kN = tc_n(C);
  constexpr int kPS = tc_psi_stride(C);
  constexpr int h = C / 2;
  const int n = P.n, H = n / 2 + 1, K = 2 * n, n_psi = P.n_psi;
  const size_t a_bytes = (size_t)kTcM * K * 2, b_bytes = (size_t)kN * K * 2;
  unsigned char* sA = smem_raw;                                  // [2][kTcM x K] fp16: hi, lo
  unsigned char* sB = sA + 2 * a_bytes;                          // [2][kN x K] fp16: hi, lo
  float2* s_p = reinterpret_cast<float2*>(sB + 2 * b_bytes);    // [kTcPsi][n] particle column
  float2* s_twr = s_p + kTcPsi * n;                              // [n]
  float2* s_twc = s_twr + n;                                     // [2][16] column twiddles times 2^-26
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_twc + 32);
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(s_bar + 2);
  int* s_slot = reinterpret_cast<int*>(s_taddr + 4);             // [kTcM] template slot (-1 = empty row)
  int* s_cand = s_slot + kTcM;                                   // [kTcM] candidate of the row

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int t = tid; t < n; t += blockDim.x) s_twr[t] = P.tw_row[t];
  for (size_t t = tid; t < 2 * b_bytes / 16; t += blockDim.x)
    reinterpret_cast<uint4*>(sB)[t] = make_uint4(0, 0, 0, 0);  // unused B rows stay zero
  if (tid == 0) {
    mbar_init(s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_taddr)),
                 "r"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t taddr = *s_taddr;
  const uint32_t idesc = make_idesc(kTcM, kN);
  const int n_pass = P.split ? 3 : 1;
  const int parts = P.split ? 2 : 1;
  uint32_t n_waited = 0, n_committed = 0;
  bool ok = true;

  // epilogue role: TMEM lane quarter q (warp % 4 by the tcgen05.ld rule), psi
  const int q = warp & 3, my_psi = warp >> 2;
  const int my_row = 32 * q + lane;
  const int n_groups = (n_psi + kTcPsi - 1) / kTcPsi;

  for (int wi = blockIdx.x; wi < P.n_work; wi += gridDim.x) {
    const int b = P.work[2 * wi], tile = P.work[2 * wi + 1] / n_groups;
    const int psi0 = (P.work[2 * wi + 1] - tile * n_groups) * kTcPsi;
    const int g_psi = min(kTcPsi, n_psi - psi0);  // psi angles in this group
    const int jrows = g_psi * kPS;
    const int e0 = P.local_ptr[b], d = P.local_ptr[b + 1] - e0;
    const int rows_total = d * P.n_cand;
    for (int m = tid; m < kTcM; m += blockDim.x) {
      const int row = tile * kTcM + m;
      if (row < rows_total) {
        const int a = row / P.n_cand;
        s_slot[m] = P.local_idx[e0 + a];
        s_cand[m] = row - a * P.n_cand;
      } else {
        s_slot[m] = -1;
        s_cand[m] = 0;
      }
    }
    __syncthreads();
    float acc[C][C];
#pragma unroll
    for (int yi = 0; yi < C; ++yi)
#pragma unroll
      for (int xi = 0; xi < C; ++xi) acc[yi][xi] = 0.f;
    const float2* Pb = P.stack + (size_t)b * n_psi * n * H;

    for (int col = 0; col <= H; ++col) {
      if (col > 0) {
        // MMA(col-1) done: shared operands are free and its TMEM buffer is final
        const bool done = mbar_wait(s_bar, n_waited & 1u);
        ++n_waited;
        ok = __syncthreads_and(done ? 1 : 0) != 0;
        if (!ok) break;
      }
      if (col < H) {
        // ---- A: the rows' template columns (fp16 hi, lo), 16-byte async copies.
        // Eight consecutive threads fill one 128-byte core matrix (conflict-free),
        // four core matrices along K per warp (64 contiguous bytes per row).
        const int chunks = K / 8;
        const int total = parts * kTcM * chunks;
        for (int t = tid; t < total; t += blockDim.x) {
          const int m_lo = t & 7, kc_lo = (t >> 3) & 3;
          int rest = t >> 5;
          const int kc_hi = rest % (chunks / 4);
          rest /= (chunks / 4);
          const int m_hi = rest % (kTcM / 8), part = rest / (kTcM / 8);
          const int m = m_hi * 8 + m_lo, kc = kc_hi * 4 + kc_lo;
          unsigned char* dst = sA + part * a_bytes + core_off(m, kc * 8, K);
          const int slot = s_slot[m];
          if (slot >= 0) {
            const __half* src = P.tbank + (size_t)s_cand[m] * (size_t)P.cand_stride +
                                (((size_t)slot * H + col) * 2 + part) * K + kc * 8;
            cp_async16(dst, src);
          } else {
            *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
          }
        }
        asm volatile("cp.async.commit_group;");
        for (int t = tid; t < g_psi * n; t += blockDim.x) {
          const int s = t / n, r = t - s * n;
          s_p[t] = __ldg(Pb + ((size_t)(psi0 + s) * n + r) * H + col);
        }
        if (tid < C) {
          const float2 e = P.tw_col[(size_t)col * C + tid];
          s_twc[(col & 1) * 16 + tid] = make_float2(e.x * kTcUnscale, e.y * kTcUnscale);
        }
        __syncthreads();
        // ---- B: U_{s,y}(r) = P_s(r, col) w^{r y}, scaled and split. A warp
        // covers 8 rows j x 8 values of r, so its half2 stores hit 32 banks.
        const int rchunks = n / 8, jgroups = (jrows + 7) / 8;
        const int btotal = jgroups * rchunks * 32;
        for (int t = tid; t < btotal; t += blockDim.x) {
          const int ln = t & 31, g = t >> 5;
          const int jg = g % jgroups, rc = g / jgroups;
          const int j = jg * 8 + (ln >> 2);
          const int s = j / kPS, jj = j - s * kPS;
          if (s >= g_psi || jj >= 2 * C) continue;
          const int yi = jj >> 1, part = jj & 1, y = yi - h;
          const int r = rc * 8 + (ln & 3) * 2;
          int i0 = (r * y) % n;
          if (i0 < 0) i0 += n;
          int i1 = i0 + y;
          if (i1 < 0) i1 += n;
          if (i1 >= n) i1 -= n;
          const float2 u0 = cscale(cmul(s_p[s * n + r], s_twr[i0]), kTcScale);
          const float2 u1 = cscale(cmul(s_p[s * n + r + 1], s_twr[i1]), kTcScale);
          // part 0 row: [Re U | -Im U]; part 1 row: [Im U | Re U]
          const float f0 = part ? u0.y : u0.x, f1 = part ? u1.y : u1.x;
          const float g0 = part ? u0.x : -u0.y, g1 = part ? u1.x : -u1.y;
          __half2 hi, lo;
          split2(f0, f1, hi, lo);
          const uint32_t o1 = core_off(j, r, K), o2 = core_off(j, n + r, K);
          st_half2(sB + o1, hi);
          if (P.split) st_half2(sB + b_bytes + o1, lo);
          split2(g0, g1, hi, lo);
          st_half2(sB + o2, hi);
          if (P.split) st_half2(sB + b_bytes + o2, lo);
        }
        asm volatile("cp.async.wait_all;");
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        // ---- stage 1 on the tensor cores: hi*hi [+ hi*lo + lo*hi]
        if (tid == 0) {
          const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
          const uint32_t sbo = (uint32_t)(K / 8) * 128;
          const uint32_t dt = taddr + (uint32_t)((col & 1) * kN);
          uint32_t acc_in = 0;
          for (int pass = 0; pass < n_pass; ++pass) {
            const uint32_t ap = a0 + (pass == 2 ? (uint32_t)a_bytes : 0u);
            const uint32_t bp = b0 + (pass == 1 ? (uint32_t)b_bytes : 0u);
            for (int ks = 0; ks < K / 16; ++ks) {
              const uint64_t ad = make_desc(ap + ks * 256, 128, sbo);
              const uint64_t bd = make_desc(bp + ks * 256, 128, sbo);
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(acc_in));
              acc_in = 1;
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(s_bar)));
        }
        ++n_committed;
      }
      if (col > 0) {
        // ---- stage 2 for column col-1 while the tensor cores run column col
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (my_psi < g_psi) {
          const int pc = col - 1;
          const uint32_t ta = taddr + ((uint32_t)(32 * q) << 16) + (uint32_t)((pc & 1) * kN + my_psi * kPS);
          const float2* twc = s_twc + (pc & 1) * 16;
          uint32_t v[8];
#pragma unroll
          for (int yg = 0; yg < C / 4; ++yg) {
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                           "=r"(v[7])
                         : "r"(ta + 8 * yg));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            stage2_rows<C, 4>(acc, v, 4 * yg, twc);
          }
          if constexpr (C % 4 == 2) {
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                         : "r"(ta + 8 * (C / 4)));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            stage2_rows<C, 2>(acc, v, 4 * (C / 4), twc);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
      }
    }
    if (!ok) break;
    // ---- first maximum of this (row, psi) map, row-major over (y, x)
    const int row = tile * kTcM + my_row;
    if (my_psi < g_psi && row < rows_total) {
      float best = -INFINITY;
      int bi = 0;
#pragma unroll
      for (int yi = 0; yi < C; ++yi)
#pragma unroll
        for (int xi = 0; xi < C; ++xi)
          if (acc[yi][xi] > best) {
            best = acc[yi][xi];
            bi = yi * C + xi;
          }
      const int a = row / P.n_cand, cand = row - a * P.n_cand;
      const size_t o = (size_t)cand * P.nnz * n_psi + (size_t)(e0 + a) * n_psi + psi0 + my_psi;
      P.out_score[o] = best * 1024.0f;
      P.out_y[o] = bi / C;
      P.out_x[o] = bi % C;
    }
    __syncthreads();  // column twiddles and TMEM buffers are reused by the next item
  }
  if (!ok) {
    if (tid == 0 && P.status != nullptr) atomicExch(P.status, 1);
    // give the MMA in flight a last bounded chance to retire before TMEM is freed
    if (n_committed > n_waited) mbar_wait(s_bar, n_waited & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTcTmemCols));
  }
}

// fp16 hi/lo copy of template banks, column-major and scaled:
// out[c][slot][col][part][k], k < n: Re T(k, col), k >= n: Im T(k - n, col).
// One block per (slot, candidate), transposed through shared memory.
__global__ void bank_to_fp16(const float2* __restrict__ bank, long long bank_stride, int n,
                             __half* __restrict__ out, long long out_stride) {
  extern __shared__ float2 s_t[];  // [n][H]
  const int H = n / 2 + 1, K = 2 * n;
  const int slot = blockIdx.x, cand = blockIdx.y;
  const float2* src = bank + (size_t)cand * (size_t)bank_stride + (size_t)slot * n * H;
  __half* dst = out + (size_t)cand * (size_t)out_stride + (size_t)slot * H * 2 * K;
  for (int t = threadIdx.x; t < n * H; t += blockDim.x) s_t[t] = src[t];
  __syncthreads();
  for (int t = threadIdx.x; t < H * (n / 2); t += blockDim.x) {
    const int col = t / (n / 2), r = (t - col * (n / 2)) * 2;
    const float2 v0 = cscale(s_t[r * H + col], kTcScale), v1 = cscale(s_t[(r + 1) * H + col], kTcScale);
    __half2 hi, lo;
    __half* base = dst + (size_t)col * 2 * K;
    split2(v0.x, v1.x, hi, lo);
    *reinterpret_cast<__half2*>(base + r) = hi;
    *reinterpret_cast<__half2*>(base + K + r) = lo;
    split2(v0.y, v1.y, hi, lo);
    *reinterpret_cast<__half2*>(base + n + r) = hi;
    *reinterpret_cast<__half2*>(base + K + n + r) = lo;
  }
}

template <int C>
cudaError_t launch_tc_c(const TcParams& P, size_t smem, int grid, cudaStream_t st) {
  static size_t set_smem = 0;
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(correlate_tc<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  correlate_tc<C><<<grid, kTcThreads, smem, st>>>(P);
  return cudaGetLastError();
}

}  // namespace

int correlate_tc_max_psi() { return kTcPsi; }
int correlate_tc_max_n() { return kTcMaxN; }

size_t correlate_tc_smem_bytes(int n, int crop) {
  const size_t K = 2 * (size_t)n;
  return 2 * (size_t)kTcM * K * 2 + 2 * (size_t)tc_n(crop) * K * 2 + (size_t)kTcPsi * n * sizeof(float2) +
         (size_t)n * sizeof(float2) + 32 * sizeof(float2) + 16 + 16 + 2 * kTcM * sizeof(int);
}

// halves in the fp16 hi/lo bank copy of one candidate
long long correlate_tc_bank_halves(int n_slot, int n) {
  return (long long)n_slot * (n / 2 + 1) * 2 * (2LL * n);
}

// Work list (particle, tile * n_groups + psi group) for the tensor-core
// kernel, sorted by the slot of the tile's first direction (then particle),
// so CTAs running at the same time read the same template columns. Host
// arrays; returns the item count.
int correlate_tc_plan(const int* local_ptr, const int* local_idx, int n_particles, int n_cand, int n_psi,
                      int* work, int max_work) {
  struct Item { int key, b, tile; };
  const int n_groups = (n_psi + kTcPsi - 1) / kTcPsi;
  std::vector<Item> items;
  for (int b = 0; b < n_particles; ++b) {
    const int e0 = local_ptr[b], d = local_ptr[b + 1] - e0;
    const long long rows = (long long)d * n_cand;
    const int tiles = (int)((rows + kTcM - 1) / kTcM);
    for (int t = 0; t < tiles; ++t) {
      const int a = (int)(((long long)t * kTcM) / n_cand);
      for (int g = 0; g < n_groups; ++g) items.push_back({local_idx[e0 + a], b, t * n_groups + g});
    }
  }
  std::stable_sort(items.begin(), items.end(), [](const Item& x, const Item& y) { return x.key < y.key; });
  const int count = (int)items.size();
  if (work != nullptr) {
    for (int i = 0; i < count && i < max_work; ++i) {
      work[2 * i] = items[i].b;
      work[2 * i + 1] = items[i].tile;
    }
  }
  return count;
}

cudaError_t launch_bank_to_fp16(cudaStream_t st, const float2* bank, long long bank_stride, int n_cand, int n_slot,
                                int n, void* out) {
  if (n_cand <= 0 || n_slot <= 0) return cudaSuccess;
  const size_t smem = (size_t)n * (n / 2 + 1) * sizeof(float2);
  static size_t set_smem = 0;
  if (set_smem < smem) {
    cudaError_t e = cudaFuncSetAttribute(bank_to_fp16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  bank_to_fp16<<<dim3(n_slot, n_cand), 256, smem, st>>>(bank, bank_stride, n, (__half*)out,
                                                         correlate_tc_bank_halves(n_slot, n));
  return cudaGetLastError();
}

cudaError_t launch_correlate_tc(cudaStream_t st, const void* tbank, int n_slot, int n_cand, const float2* stack,
                                const int* local_ptr, const int* local_idx, const int* work, int n_work, int n_psi,
                                int n, int crop, int nnz, int split, const float2* tw_row, const float2* tw_col,
                                float* out_score, int* out_y, int* out_x, int* status, int grid) {
  if (n_work <= 0 || n_cand <= 0) return cudaSuccess;
  TcParams P;
  P.tbank = (const __half*)tbank;
  P.cand_stride = correlate_tc_bank_halves(n_slot, n);
  P.stack = stack;
  P.local_ptr = local_ptr;
  P.local_idx = local_idx;
  P.work = work;
  P.n_work = n_work;
  P.n_cand = n_cand;
  P.n_psi = n_psi;
  P.n = n;
  P.nnz = nnz;
  P.split = split ? 1 : 0;
  P.tw_row = tw_row;
  P.tw_col = tw_col;
  P.out_score = out_score;
  P.out_y = out_y;
  P.out_x = out_x;
  P.status = status;
  const size_t smem = correlate_tc_smem_bytes(n, crop);
  switch (crop) {
    case 2: return launch_tc_c<2>(P, smem, grid, st);
    case 4: return launch_tc_c<4>(P, smem, grid, st);
    case 6: return launch_tc_c<6>(P, smem, grid, st);
    case 8: return launch_tc_c<8>(P, smem, grid, st);
    case 10: return launch_tc_c<10>(P, smem, grid, st);
    case 12: return launch_tc_c<12>(P, smem, grid, st);
    default: return cudaErrorInvalidValue;
  }
}
