// Tensor-core correlation for batches of candidates (tcgen05, TMEM), sm_103a.
//
// The crop-window transform of the plain kernel is, per packed column c,
//     Z_{m,s}(y, c) = sum_r T_m(r, c) * P_s(r, c) * w_n^{r y}          (stage 1)
//     raw_{m,s}(y, x) = sum_c Re[Z_{m,s}(y, c) w_c w_n^{c x}]         (stage 2)
// for rows m = (local direction, candidate) of one particle and its psi
// angles s. For a fixed particle and column, stage 1 is a complex GEMM
// between the rows' template columns T_m(., c) and U_{s,y}(r) = P_s(r,c) w^{ry},
// shared by every candidate: in real form D[m][j] = sum_k A[m][k] B[j][k] with
// A = [Re T | Im T] and B's row j = (s, y, part) holding [Re U | -Im U]
// (part 0, Re Z) or [Im U | Re U] (part 1, Im Z). K (2n) is split into two
// halves by row r (r < n/2, r >= n/2), each holding [Re | Im] of its rows.
//
// Precision: both operands are scaled by 2^13 (every entry has modulus <= 1,
// the packed spectra having unit L2 norm) and split into fp16 hi + lo parts;
// the split form accumulates hi*hi + hi*lo + lo*hi in FP32 (three passes of
// tcgen05.mma), which keeps about 22 significant bits per product. The single
// form uses hi*hi only.
//
// Work item: one particle, a tile of whole directions x all candidates
// (row = direction_in_tile * n_cand + cand, n_cand <= 128) and a group of up
// to three psi angles; the work list is sorted by direction so CTAs running
// together share template columns in L2. Per column and K half, one lane
// group of warp 0 issues bulk async copies of the rows' template chunks (the
// fp16 bank copy is laid out [slot][col][half][part][k/8][cand][8], so each
// direction's chunk is contiguous) into a two-stage shared-memory ring, all
// warps build B for that half, and one thread issues the MMAs into one of two
// TMEM accumulators (M=128, N=kN, K=16) and commits to mbarriers. The MMAs of
// one half overlap the B build of the next; twelve warps read the previous
// column from TMEM (tcgen05.ld) and accumulate stage 2 with packed FP32 FMAs
// in registers; after the last column each thread takes the row-major first
// maximum of its (row, psi) map. Operands use the K-major no-swizzle layout
// with core matrices (8 rows x 16 bytes) stored K-chunk-major: SBO = 128 B
// between 8-row groups, LBO = rows * 16 B between K chunks. Every mbarrier
// wait is bounded; on timeout the kernel sets *status, waits (bounded) for
// the MMAs in flight, frees TMEM and returns.
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kTcThreads = 384;   // 12 warps: 3 per TMEM lane quarter
constexpr int kTcM = 128;         // rows per tile (TMEM lanes)
constexpr int kTcPsi = 3;         // psi angles per particle held by a tile
constexpr int kTcMaxN = 128;      // half of K = n <= 128 per stage
constexpr int kTcMaxCand = 128;   // candidates per launch
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
  const __half* tbank;    // [n_slot][H][2 halves][2 parts][n/8][n_cand][8], scaled
  const float2* stack;    // [n_particles][n_psi][n][H]
  const int* local_ptr;
  const int* local_idx;
  const int* work;        // [n_work][2]: particle, tile * n_groups + psi group
  int n_work, n_cand, n_psi, n, nnz, split, dpt;  // dpt: directions per tile
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

// tcgen05 shared-memory matrix descriptor, no swizzle (K-major core matrices):
// lbo = byte step between core matrices along K, sbo = between 8-row groups.
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes));
}

// contiguous global -> shared copy on the async proxy, completion counted in bytes on bar
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)));
}

// fp16 hi/lo of 8 floats as 4 half2 words each
__device__ __forceinline__ void split8(const float (&v)[8], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __half2 a = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    const float2 af = __half22float2(a);
    const __half2 b = __floats2half2_rn(v[2 * i] - af.x, v[2 * i + 1] - af.y);
    h[i] = *reinterpret_cast<const uint32_t*>(&a);
    l[i] = *reinterpret_cast<const uint32_t*>(&b);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ uint4 neg8(uint4 v) {
  return make_uint4(v.x ^ 0x80008000u, v.y ^ 0x80008000u, v.z ^ 0x80008000u, v.w ^ 0x80008000u);
}

// Accumulate stage 2 for the crop-row pair yp from a TMEM load of
// (Re Z(2yp), Re Z(2yp+1), Im Z(2yp), Im Z(2yp+1)):
// acc[yp][x] += (Re Z pair) * Er(x) - (Im Z pair) * Ei(x), with the twiddles
// stored pre-broadcast as (Er, Er, -Ei, -Ei).
// The twiddle loads are volatile so that they are not hoisted out of the
// crop-row loop (that would hold 4 C more registers next to the accumulators).
__device__ __forceinline__ float4 lds_v4(uint32_t addr) {
  float4 r;
  asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "r"(addr));
  return r;
}

template <int C>
__device__ __forceinline__ void stage2_pair(float2 (&acc)[C / 2][C], const uint32_t (&v)[4], int yp,
                                            uint32_t tw) {
  const float2 zr = make_float2(__uint_as_float(v[0]), __uint_as_float(v[1]));
  const float2 zi = make_float2(__uint_as_float(v[2]), __uint_as_float(v[3]));
#pragma unroll
  for (int x = 0; x < C; ++x) {
    const float4 e = lds_v4(tw + 16 * x);
    acc[yp][x] = __ffma2_rn(zi, make_float2(e.z, e.w), acc[yp][x]);
    acc[yp][x] = __ffma2_rn(zr, make_float2(e.x, e.y), acc[yp][x]);
  }
}

template <int C>
__global__ void __launch_bounds__(kTcThreads, 1) correlate_tc(TcParams P) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  static_assert(C % 2 == 0 && C <= 12, "even crop up to 12");
  constexpr int kN = tc_n(C);
  constexpr int kPS = tc_psi_stride(C);
  constexpr int h = C / 2;
  const int n = P.n, H = n / 2 + 1, n_psi = P.n_psi, n_cand = P.n_cand;
  const int kc_n = n / 8;                                      // 16-byte K chunks per half
  const uint32_t a_part = (uint32_t)kc_n * kTcM * 16;          // bytes of A (hi or lo) per stage
  const uint32_t lbo_b = kN * 16 + 16;                         // B chunk stride, padded so chunks spread banks
  const uint32_t b_part = (uint32_t)kc_n * lbo_b;
  const uint32_t stage_bytes = 2 * a_part + 2 * b_part;
  unsigned char* stages = smem_raw;                            // [2][A hi, A lo, B hi, B lo]
  float2* s_p = reinterpret_cast<float2*>(smem_raw + 2 * stage_bytes);  // [kTcPsi][n] scaled column
  float2* s_twr = s_p + kTcPsi * n;                            // [n]
  float4* s_twc = reinterpret_cast<float4*>(s_twr + n);        // [2][16] (Er, Er, -Ei, -Ei) times 2^-26
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_twc + 32);   // full[2], empty[2], tmem[2]
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(s_bar + 6);
  int* s_fail = reinterpret_cast<int*>(s_taddr + 1);
  int* s_slot = s_fail + 1;                                    // [kTcM] template slot per tile direction
  uint64_t* bar_full = s_bar;
  uint64_t* bar_empty = s_bar + 2;
  uint64_t* bar_tmem = s_bar + 4;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int t = tid; t < n; t += blockDim.x) s_twr[t] = P.tw_row[t];
  for (uint32_t t = tid; t < 2 * stage_bytes / 16; t += blockDim.x)
    reinterpret_cast<uint4*>(stages)[t] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    for (int i = 0; i < 6; ++i) mbar_init(s_bar + i, 1);
    *s_fail = 0;
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
  const int parts = P.split ? 2 : 1;
  const int n_pass = P.split ? 3 : 1;
  uint32_t uses[2] = {0, 0};        // commits issued per stage (one per use)
  uint32_t tmem_waits[2] = {0, 0};  // completions consumed per TMEM buffer
  bool ok = true;

  // epilogue role: TMEM lane quarter q (warp % 4 by the tcgen05.ld rule), psi
  const int q = warp & 3, my_psi = warp >> 2;
  const int my_row = 32 * q + lane;
  const int n_groups = (n_psi + kTcPsi - 1) / kTcPsi;
  int zeroed_from = kTcM;  // rows [zeroed_from, 128) of A are zero in both stages

  for (int wi = blockIdx.x; wi < P.n_work && ok; wi += gridDim.x) {
    const int b = P.work[2 * wi], tile = P.work[2 * wi + 1] / n_groups;
    const int psi0 = (P.work[2 * wi + 1] - tile * n_groups) * kTcPsi;
    const int g_psi = min(kTcPsi, n_psi - psi0);  // psi angles in this group
    const int e0 = P.local_ptr[b], d = P.local_ptr[b + 1] - e0;
    const int a0 = tile * P.dpt, nd = min(P.dpt, d - a0);
    const int used = nd * n_cand;
    if (tid < nd) s_slot[tid] = P.local_idx[e0 + a0 + tid];
    if (used < zeroed_from) {
      // rows this tile leaves empty must read as zero (no MMA is in flight here)
      const int nz = zeroed_from - used;  // rows [used, zeroed_from) per K chunk
      const int per_chunk = nz;           // 16-byte rows per (stage, part, chunk)
      const int total = 2 * 2 * kc_n * per_chunk;
      for (int t = tid; t < total; t += blockDim.x) {
        const int row = used + t % per_chunk;
        const int rest = t / per_chunk;
        const int kc = rest % kc_n, sp = rest / kc_n;  // sp = stage * 2 + part
        unsigned char* base = stages + (sp >> 1) * stage_bytes + (sp & 1) * a_part;
        *reinterpret_cast<uint4*>(base + (size_t)kc * kTcM * 16 + row * 16) = make_uint4(0, 0, 0, 0);
      }
      asm volatile("fence.proxy.async.shared::cta;");
    }
    zeroed_from = used;
    __syncthreads();
    const int jrows = g_psi * kPS;
    const int b_tasks = g_psi * C * (n / 16);  // (psi, y, 8-row chunk) per half
    float2 acc[C / 2][C];  // .x: crop row 2yp, .y: crop row 2yp + 1
#pragma unroll
    for (int yp = 0; yp < C / 2; ++yp)
#pragma unroll
      for (int x = 0; x < C; ++x) acc[yp][x] = make_float2(0.f, 0.f);
    const float2* Pb = P.stack + ((size_t)b * n_psi + psi0) * n * H;
    (void)jrows;

    for (int col = 0; col <= H && ok; ++col) {
      if (col < H) {
        for (int hh = 0; hh < 2; ++hh) {
          unsigned char* stA = stages + hh * stage_bytes;
          unsigned char* stB = stA + 2 * a_part;
          if (uses[hh] > 0) {
            // the MMAs that last read this stage are done
            const bool done = mbar_wait(bar_empty + hh, (uses[hh] - 1) & 1u);
            ok = __syncthreads_and(done ? 1 : 0) != 0;
            if (!ok) break;
          }
          // ---- A: one bulk copy per (part, K chunk, direction), n_cand rows of 16 B
          if (warp == 0) {
            const uint32_t chunk = (uint32_t)n_cand * 16;
            if (lane == 0) mbar_expect_tx(bar_full + hh, (uint32_t)(parts * kc_n * nd) * chunk);
            __syncwarp();
            for (int qd = lane; qd < parts * kc_n * nd; qd += 32) {
              const int part = qd / (kc_n * nd), rem = qd - part * (kc_n * nd);
              const int kc = rem / nd, dl = rem - kc * nd;
              const __half* src = P.tbank + ((((size_t)s_slot[dl] * H + col) * 2 + hh) * 2 + part) *
                                                (size_t)kc_n * n_cand * 8 +
                                  (size_t)kc * n_cand * 8;
              bulk_copy(stA + part * a_part + (uint32_t)kc * kTcM * 16 + (uint32_t)dl * chunk, src, chunk,
                        bar_full + hh);
            }
          }
          if (hh == 0) {
            for (int t = tid; t < g_psi * n; t += blockDim.x) {
              const int s = t / n, r = t - s * n;
              s_p[t] = cscale(__ldg(Pb + ((size_t)s * n + r) * H + col), kTcScale);
            }
            if (tid < C) {
              const float2 e = P.tw_col[(size_t)col * C + tid];
              const float er = e.x * kTcUnscale, ei = -e.y * kTcUnscale;
              s_twc[(col & 1) * 16 + tid] = make_float4(er, er, ei, ei);
            }
            __syncthreads();
          }
          // ---- B for this half: rows r in [hh n/2, hh n/2 + n/2), chunk kc < n/16 holds
          // Re (part-0 row) / Im (part-1 row), chunk n/16 + kc holds -Im / Re
          for (int t = tid; t < b_tasks; t += blockDim.x) {
            const int yi = t % C, rest = t / C;
            const int s = rest % g_psi, rc = rest / g_psi;
            const int y = yi - h;
            const int r0 = hh * (n / 2) + rc * 8;
            float2 tw = s_twr[(r0 * y) & (n - 1)];
            const float2 step = s_twr[y & (n - 1)];
            float re[8], im[8];
            const float2* pp = s_p + s * n + r0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const float2 u = cmul(pp[i], tw);
              re[i] = u.x;
              im[i] = u.y;
              tw = cmul(tw, step);
            }
            // rows of psi s: per crop-row pair (Re y, Re y+1, Im y, Im y+1)
            const int jr = s * kPS + 4 * (yi >> 1) + (yi & 1), ji = jr + 2;
            unsigned char* c_re = stB + (uint32_t)rc * lbo_b;
            unsigned char* c_im = stB + (uint32_t)(n / 16 + rc) * lbo_b;
            uint4 hi, lo;
            split8(re, hi, lo);  // Re U: Re-Z row first half, Im-Z row second half
            *reinterpret_cast<uint4*>(c_re + jr * 16) = hi;
            *reinterpret_cast<uint4*>(c_im + ji * 16) = hi;
            if (P.split) {
              *reinterpret_cast<uint4*>(c_re + b_part + jr * 16) = lo;
              *reinterpret_cast<uint4*>(c_im + b_part + ji * 16) = lo;
            }
            split8(im, hi, lo);  // Im U: Im-Z row first half, negated in the Re-Z row second half
            *reinterpret_cast<uint4*>(c_re + ji * 16) = hi;
            *reinterpret_cast<uint4*>(c_im + jr * 16) = neg8(hi);
            if (P.split) {
              *reinterpret_cast<uint4*>(c_re + b_part + ji * 16) = lo;
              *reinterpret_cast<uint4*>(c_im + b_part + jr * 16) = neg8(lo);
            }
          }
          asm volatile("fence.proxy.async.shared::cta;");
          asm volatile("tcgen05.fence::before_thread_sync;");
          __syncthreads();
          asm volatile("tcgen05.fence::after_thread_sync;");
          // ---- stage 1 on the tensor cores: hi*hi [+ hi*lo + lo*hi] over this half
          if (tid == 0) {
            if (!mbar_wait(bar_full + hh, uses[hh] & 1u)) {
              *s_fail = 1;
            } else {
              asm volatile("tcgen05.fence::after_thread_sync;");
              const uint32_t a0s = smem_u32(stA), b0s = smem_u32(stB);
              const uint32_t dt = taddr + (uint32_t)((col & 1) * kN);
              const uint32_t lbo_a = kTcM * 16;
              uint32_t acc_in = hh;
              for (int pass = 0; pass < n_pass; ++pass) {
                const uint32_t ap = a0s + (pass == 2 ? a_part : 0u);
                const uint32_t bp = b0s + (pass == 1 ? b_part : 0u);
                for (int ks = 0; ks < kc_n / 2; ++ks) {
                  const uint64_t ad = make_desc(ap + (uint32_t)ks * 2 * lbo_a, lbo_a, 128);
                  const uint64_t bd = make_desc(bp + (uint32_t)ks * 2 * lbo_b, lbo_b, 128);
                  asm volatile(
                      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
                      "l"(ad), "l"(bd), "r"(idesc), "r"(acc_in));
                  acc_in = 1;
                }
              }
              mma_commit(bar_empty + hh);
              if (hh == 1) mma_commit(bar_tmem + (col & 1));
            }
          }
          ++uses[hh];
        }
        if (!ok) break;
      }
      if (col > 0) {
        // ---- stage 2 for column col-1 while the tensor cores run column col
        const int pb = (col - 1) & 1;
        const bool done = mbar_wait(bar_tmem + pb, tmem_waits[pb] & 1u);
        ++tmem_waits[pb];
        ok = __syncthreads_and((done && *s_fail == 0) ? 1 : 0) != 0;
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (my_psi < g_psi) {
          const uint32_t ta = taddr + ((uint32_t)(32 * q) << 16) + (uint32_t)(pb * kN + my_psi * kPS);
          const uint32_t tw = smem_u32(s_twc + pb * 16);
          uint32_t v[4];
#pragma unroll
          for (int yp = 0; yp < C / 2; ++yp) {
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                         : "r"(ta + 4 * yp));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            stage2_pair<C>(acc, v, yp, tw);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
      }
    }
    if (!ok) break;
    // ---- first maximum of this (row, psi) map, row-major over (y, x)
    if (my_psi < g_psi && my_row < used) {
      float best = -INFINITY;
      int bi = 0;
#pragma unroll
      for (int yp = 0; yp < C / 2; ++yp) {
#pragma unroll
        for (int x = 0; x < C; ++x)
          if (acc[yp][x].x > best) {
            best = acc[yp][x].x;
            bi = 2 * yp * C + x;
          }
#pragma unroll
        for (int x = 0; x < C; ++x)
          if (acc[yp][x].y > best) {
            best = acc[yp][x].y;
            bi = (2 * yp + 1) * C + x;
          }
      }
      const int dl = my_row / n_cand, cand = my_row - dl * n_cand;
      const size_t o = (size_t)cand * P.nnz * n_psi + (size_t)(e0 + a0 + dl) * n_psi + psi0 + my_psi;
      P.out_score[o] = best * 1024.0f;
      P.out_y[o] = bi / C;
      P.out_x[o] = bi % C;
    }
    __syncthreads();  // column twiddles, slots and TMEM buffers are reused by the next item
  }
  if (!ok) {
    if (tid == 0 && P.status != nullptr) atomicExch(P.status, 1);
    // give MMAs still in flight a last bounded chance to retire before TMEM is freed
    for (int s = 0; s < 2; ++s)
      if (uses[s] > 0) mbar_wait(bar_empty + s, (uses[s] - 1) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTcTmemCols));
  }
}

// fp16 hi/lo copy of template banks for the tensor-core kernel:
// out[slot][col][half][part][k/8][cand][k%8] with, per half hh, k < n/2 the
// real part and k >= n/2 the imaginary part of rows r = hh n/2 + (k mod n/2),
// scaled by 2^13. One block per (slot, candidate), transposed through shared
// memory; every thread writes whole 16-byte chunks.
__global__ void bank_to_fp16(const float2* __restrict__ bank, long long bank_stride, int n, int n_cand,
                             __half* __restrict__ out) {
  extern __shared__ float2 s_t[];  // [n][H]
  const int H = n / 2 + 1, kc_n = n / 8;
  const int slot = blockIdx.x, cand = blockIdx.y;
  const float2* src = bank + (size_t)cand * (size_t)bank_stride + (size_t)slot * n * H;
  for (int t = threadIdx.x; t < n * H; t += blockDim.x) s_t[t] = src[t];
  __syncthreads();
  // one task per (col, half, K chunk): 8 consecutive k -> hi and lo chunks
  for (int t = threadIdx.x; t < H * 2 * kc_n; t += blockDim.x) {
    const int kc = t % kc_n, hh = (t / kc_n) % 2, col = t / (2 * kc_n);
    const bool imag = kc >= kc_n / 2;
    const int r0 = hh * (n / 2) + (kc % (kc_n / 2)) * 8;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float2 z = s_t[(r0 + i) * H + col];
      v[i] = (imag ? z.y : z.x) * kTcScale;
    }
    uint4 hi, lo;
    split8(v, hi, lo);
    const size_t base = ((((size_t)slot * H + col) * 2 + hh) * 2) * kc_n;  // part 0 chunk index
    *reinterpret_cast<uint4*>(out + ((base + kc) * n_cand + cand) * 8) = hi;
    *reinterpret_cast<uint4*>(out + ((base + kc_n + kc) * n_cand + cand) * 8) = lo;
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
int correlate_tc_max_cand() { return kTcMaxCand; }

size_t correlate_tc_smem_bytes(int n, int crop) {
  const size_t kc_n = (size_t)n / 8;
  const size_t stage = 2 * kc_n * kTcM * 16 + 2 * kc_n * ((size_t)tc_n(crop) * 16 + 16);
  return 2 * stage + (size_t)kTcPsi * n * sizeof(float2) + (size_t)n * sizeof(float2) + 32 * sizeof(float4) +
         6 * 8 + 8 + (size_t)kTcM * sizeof(int);
}

// halves in the fp16 hi/lo bank copy of one candidate
long long correlate_tc_bank_halves(int n_slot, int n) {
  return (long long)n_slot * (n / 2 + 1) * 2 * (2LL * n);
}

// directions per tile for a launch of n_cand candidates
int correlate_tc_dirs_per_tile(int n_cand) { return n_cand > 0 ? kTcM / std::min(n_cand, kTcMaxCand) : 0; }

// Work list (particle, tile * n_groups + psi group) for the tensor-core
// kernel, sorted by the slot of the tile's first direction (then particle),
// so CTAs running at the same time read the same template columns. A tile
// holds 128 / n_cand whole directions (n_cand <= 128). Host arrays; returns
// the item count.
int correlate_tc_plan(const int* local_ptr, const int* local_idx, int n_particles, int n_cand, int n_psi,
                      int* work, int max_work) {
  struct Item { int key, b, tile; };
  const int n_groups = (n_psi + kTcPsi - 1) / kTcPsi;
  const int dpt = correlate_tc_dirs_per_tile(n_cand);
  std::vector<Item> items;
  for (int b = 0; b < n_particles; ++b) {
    const int e0 = local_ptr[b], d = local_ptr[b + 1] - e0;
    const int tiles = (d + dpt - 1) / dpt;
    for (int t = 0; t < tiles; ++t)
      for (int g = 0; g < n_groups; ++g) items.push_back({local_idx[e0 + t * dpt], b, t * n_groups + g});
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
  bank_to_fp16<<<dim3(n_slot, n_cand), 256, smem, st>>>(bank, bank_stride, n, n_cand, (__half*)out);
  return cudaGetLastError();
}

cudaError_t launch_correlate_tc(cudaStream_t st, const void* tbank, int n_cand, const float2* stack,
                                const int* local_ptr, const int* local_idx, const int* work, int n_work, int n_psi,
                                int n, int crop, int nnz, int split, const float2* tw_row, const float2* tw_col,
                                float* out_score, int* out_y, int* out_x, int* status, int grid) {
  if (n_work <= 0 || n_cand <= 0) return cudaSuccess;
  if (n_cand > kTcMaxCand) return cudaErrorInvalidValue;
  TcParams P;
  P.tbank = (const __half*)tbank;
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
  P.dpt = correlate_tc_dirs_per_tile(n_cand);
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
