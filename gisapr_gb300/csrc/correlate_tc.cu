// Tensor-core correlation for batches of candidates (tcgen05, TMEM), sm_103a.
//
// The crop-window transform of the plain kernel is, per packed column c,
//     Z_{m,s}(y, c) = sum_r T_m(r, c) * P_s(r, c) * w_n^{r y}          (stage 1)
//     raw_{m,s}(y, x) = sum_c Re[Z_{m,s}(y, c) w_c w_n^{c x}]         (stage 2)
// for rows m = (local direction, candidate) of one particle and its psi
// angles s. For a fixed particle and column, stage 1 is a complex GEMM
// between the rows' template columns T_m(., c) and U_{s,y}(r) = P_s(r,c) w^{ry},
// shared by every candidate: in real form D[m][j] = sum_k A[m][k] B[j][k]. A
// K step covers 32 rows r: its 64 K elements are [Re T of the 32 rows | Im T
// of the 32 rows], and B's rows j = (s, crop-row pair, part) hold
// [Re U | -Im U] (part 0, Re Z) or [Im U | Re U] (part 1, Im Z) on the same
// K positions.
//
// Precision. Operands are fp16 or bf16 (kind::f16 takes either, both sides
// of one MMA the same type). Both are scaled by 2^13 times a power of two per
// packed column (the template side's from the FSC weights of the column, the
// particle side's from the job's largest coefficient of the column), so that
// high-frequency columns keep fp16's normal range; stage 2 undoes the column
// scales in FP32 through its twiddle table. The split forms store hi and lo
// parts (x = hi + lo, both rounded to the operand type) and accumulate
// hi*hi + hi*lo + lo*hi in FP32 over three MMA passes; the single forms keep
// hi*hi.
//
// Work item: one particle, a tile of whole directions x all candidates
// (row = direction_in_tile * ceil8(n_cand) + cand, n_cand <= 128) and a group
// of up to three psi angles (two at crop 14); the work list is sorted by
// direction so CTAs running together share template columns in L2.
//
// Warp roles (640 threads, 20 warps): warp 0 issues the MMAs (one lane),
// warp 1 the bulk async copies (cp.async.bulk, mbarrier complete_tx) of the
// rows' template chunks into the A ring of shared-memory stages (the operand
// bank is laid out [slot][col][step][part][cand][128 B], so each
// direction's rows of a step are one contiguous copy; the rows of the column
// two ahead are prefetched into L2), warps 2-7 build B for each K step into
// the B ring from the particle column (prefetched with cp.async two columns
// ahead) and a table of twiddles, and warps 8-19 run stage 2: each
// thread owns one (row, psi) map, reads the finished column accumulator from
// TMEM (tcgen05.ld) and accumulates its crop rows, some in registers and the
// rest in free TMEM columns. Two TMEM accumulators let the MMAs of a column
// overlap stage 2 of the previous one. Operand tiles use the K-major
// 128-byte-swizzle layout (8-row atoms of 1024 B).
//
// Every mbarrier hand-off wait is bounded by a launch parameter; when one
// runs out the kernel sets *status, every role leaves its loop, the kernel
// waits (with the default bound) for the bulk copies and MMAs it issued,
// frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kTcThreads = 640;   // 20 warps (roles above)
constexpr int kTcBuildWarp0 = 2, kTcBuildWarps = 6;
constexpr int kTcBuilders = kTcBuildWarps * 32;
constexpr int kTcEpiWarp0 = 8, kTcEpiWarps = 12;
constexpr int kTcM = 128;         // rows per tile (TMEM lanes)
constexpr int kTcPsi = 3;         // psi angles per particle a tile holds at most
constexpr int kTcMaxN = 256;      // K = 2n <= 512, in steps of 64 (32 rows r)

// psi angles per tile: three up to crop 12; at crop 14 two, so that the MMA
// accumulators and the stage-2 rows kept in TMEM fit its 512 columns.
__host__ __device__ constexpr int tc_psi_group(int C) { return C <= 12 ? 3 : 2; }
// Shared-memory rings: A stages (the bulk-copied template rows of a K step)
// and B stages (the built particle rows) are separate, so the copies can run
// further ahead than the B build; their depths are launch parameters.
constexpr int kTcMaxSA = 8, kTcMaxSB = 3;
constexpr size_t kTcSmemMax = 232448;  // dynamic shared memory of one CTA (227 KB)
constexpr int kTcMaxCand = 128;   // candidates per launch
constexpr int kTcTmemCols = 512;
constexpr float kTcScale = 8192.0f;       // 2^13 on each operand (times the column scale)
constexpr unsigned kWaitLimit = 1u << 24; // default bound of a barrier wait (iterations)

// TMEM / B-row stride of one psi angle: crop x (re, im), rounded up to 8 so
// every tcgen05.ld starts on an 8-column boundary.
__host__ __device__ constexpr int tc_psi_stride(int C) { return ((2 * C + 7) / 8) * 8; }
// MMA N: all psi angles, rounded up to a multiple of 16.
__host__ __device__ constexpr int tc_n(int C) { return ((tc_psi_group(C) * tc_psi_stride(C) + 15) / 16) * 16; }
// crop rows of a stage-2 map held in registers (96 registers a thread);
// the rest live in TMEM columns after the two MMA accumulators
template <int C>
__host__ __device__ constexpr int tc_reg_rows() { return C <= 6 ? C : (C == 8 || C == 12 ? 4 : 2); }

struct TcParams {
  const void* tbank;      // [n_slot][H][NQ][2 parts][n_cand][128 B] operand bank (hi, lo)
  const float2* stack;    // [n_particles][n_psi][n][H]
  const int* local_ptr;
  const int* local_idx;
  const int* work;        // [n_work][2]: particle, tile * n_groups + psi group
  int n_work, n_cand, n_psi, n, nnz, split, bf16, dpt;  // dpt: directions per tile
  const float2* tw_row;   // [n]  exp(+2 pi i t / n)
  const float2* tw_col;   // [H][C]  w_c exp(+2 pi i c (x - h) / n)
  const float* t_scale;   // [H] per-column template scale (power of two) or null
  const float* p_scale;   // [H] per-column particle scale (power of two) or null
  unsigned wait_limit;    // bound of a hand-off wait (iterations)
  int sa, sb;             // A and B ring depths
  float* out_score;       // [n_cand][nnz][n_psi]
  int* out_y;
  int* out_x;
  int* status;            // set to 1 when a barrier wait ran out
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// kind::f16 instruction descriptor: FP32 accumulate, A and B K-major, both
// fp16 (formats 0) or both bf16 (formats 1).
__host__ __device__ constexpr uint32_t make_idesc(int M, int N, int bf16) {
  return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// Wait for the barrier phase of the given parity, at most ``limit``
// attempts; returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned limit) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < limit; ++it) {
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

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// contiguous global -> shared copy on the async proxy, completion counted in bytes on bar
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)));
}

// hi and lo words of two floats in the operand type: hi = round(a, b),
// lo = round(a - hi, b - hi)
template <bool BF>
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
  if constexpr (BF) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  } else {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
}

// sign flip of both 16-bit values (fp16 and bf16 keep the sign in bit 15)
__device__ __forceinline__ uint4 neg8(uint4 v) {
  return make_uint4(v.x ^ 0x80008000u, v.y ^ 0x80008000u, v.z ^ 0x80008000u, v.w ^ 0x80008000u);
}

// Stage 2 uses the symmetry of the crop twiddles E(c, x) = w_c e^{2 pi i c (x-h)/n}:
// E(c, h-k) = conj E(c, h+k). With A_k = sum_c Re Z Re E(c, h+k) and
// B_k = sum_c Im Z Im E(c, h+k), raw(h+k) = A_k - B_k and raw(h-k) = A_k + B_k
// for k = 1..h-1, raw(h) = A_0, and raw(0) (no partner) is accumulated
// directly. Accumulator slots per crop row: 0: A_0, 1: raw(0), 2..h: A_1..A_{h-1},
// h+1..2h-1: B_1..B_{h-1}. The per-column twiddle table (floats, 16-byte
// groups) holds Re E(h), Re E(0), -Im E(0), a pad entry, then Re E(h+k),
// Im E(h+k) for k = 1..h-1, each divided by the column's operand scales.
__host__ __device__ constexpr int tc_tw_entries(int C) { return ((C + 2 + 3) / 4) * 4; }

// The twiddle loads are volatile so that they are not hoisted out of the
// crop-row loop (that would hold the table in registers next to the
// accumulators and spill).
__device__ __forceinline__ float4 lds_v4(uint32_t addr) {
  float4 r;
  asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "r"(addr));
  return r;
}

// stage 2 for one crop row held in a[C] (Re Z = zr, Im Z = zi); tw: shared
// address of the column's twiddle table
template <int C>
__device__ __forceinline__ void stage2_row(float (&a)[C], float zr, float zi, uint32_t tw) {
  constexpr int h = C / 2;
  const float4 e = lds_v4(tw);  // Re E(h), Re E(0), -Im E(0), pad
  a[0] = fmaf(zr, e.x, a[0]);
  a[1] = fmaf(zi, e.z, fmaf(zr, e.y, a[1]));
#pragma unroll
  for (int k = 1; k < h; k += 2) {
    const float4 f = lds_v4(tw + 16 + 8 * (k - 1));  // k and k+1: Re E, Im E
    a[1 + k] = fmaf(zr, f.x, a[1 + k]);
    a[h + k] = fmaf(zi, f.y, a[h + k]);
    if (k + 1 < h) {
      a[2 + k] = fmaf(zr, f.z, a[2 + k]);
      a[h + k + 1] = fmaf(zi, f.w, a[h + k + 1]);
    }
  }
}

// TMEM load / store of one accumulator row (C 32-bit columns)
template <int C>
__device__ __forceinline__ void tmem_ld_row(float (&a)[C], uint32_t ta) {
  static_assert(C % 2 == 0 && C >= 2 && C <= 14, "even crop up to 14");
  uint32_t* r = reinterpret_cast<uint32_t*>(a);
  if constexpr (C >= 8) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(ta));
  }
  if constexpr (C == 12 || C == 4 || C == 14) {
    constexpr int o = C == 14 ? 8 : C - 4;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[o]), "=r"(r[o + 1]), "=r"(r[o + 2]), "=r"(r[o + 3])
                 : "r"(ta + o));
  }
  if constexpr (C == 10 || C == 6 || C == 2 || C == 14) {
    constexpr int o = C - 2;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[o]), "=r"(r[o + 1]) : "r"(ta + o));
  }
  if constexpr (C == 6) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(ta));
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;");
}
template <int C>
__device__ __forceinline__ void tmem_st_row(const float (&a)[C], uint32_t ta) {
  const uint32_t* r = reinterpret_cast<const uint32_t*>(a);
  if constexpr (C >= 8) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]));
  }
  if constexpr (C == 12 || C == 4 || C == 14) {
    constexpr int o = C == 14 ? 8 : C - 4;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(ta + o), "r"(r[o]),
                 "r"(r[o + 1]), "r"(r[o + 2]), "r"(r[o + 3]));
  }
  if constexpr (C == 10 || C == 6 || C == 2 || C == 14) {
    constexpr int o = C - 2;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" ::"r"(ta + o), "r"(r[o]), "r"(r[o + 1]));
  }
  if constexpr (C == 6) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(ta), "r"(r[0]), "r"(r[1]),
                 "r"(r[2]), "r"(r[3]));
  }
}

// raw(y, x) of a crop row from its accumulator slots (see stage2_row)
template <int C>
__device__ __forceinline__ float raw_at(const float (&a)[C], int x) {
  constexpr int h = C / 2;
  if (x == 0) return a[1];
  if (x == h) return a[0];
  if (x < h) return a[1 + (h - x)] + a[h + (h - x)];
  return a[1 + (x - h)] - a[h + (x - h)];
}

// Entry j of column col's stage-2 twiddle table (see stage2_row), divided by
// the column's two operand scales.
template <int C>
__device__ __forceinline__ float tw_entry(const float2* __restrict__ tw_col, int col, int j, float unscale) {
  constexpr int h = C / 2;
  const float2* e = tw_col + (size_t)col * C;
  float v = 0.f;
  if (j == 0) v = e[h].x;
  else if (j == 1) v = e[0].x;
  else if (j == 2) v = -e[0].y;
  else if (j >= 4 && j < 4 + 2 * (h - 1)) {
    const int k = 1 + (j - 4) / 2;
    v = ((j - 4) & 1) ? e[h + k].y : e[h + k].x;
  }
  return v * unscale;
}

// tcgen05 shared-memory descriptor of a 128-byte-swizzled K-major tile
// (8-row atoms of 1024 B; the leading byte offset is unused and set to 1).
__device__ __forceinline__ uint64_t make_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;             // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}

// One K step (64 elements = four MMAs of K = 16) per pass: pass 0 A_hi*B_hi,
// pass 1 A_hi*B_lo, pass 2 A_lo*B_hi; d accumulates unless first.
__device__ __forceinline__ void issue_mma_step(uint32_t d, uint32_t a0, uint32_t b0, uint32_t a_part,
                                               uint32_t b_part, uint32_t idesc, int n_pass, bool accumulate) {
  uint32_t acc_in = accumulate ? 1u : 0u;
  for (int pass = 0; pass < n_pass; ++pass) {
    const uint32_t ap = a0 + (pass == 2 ? a_part : 0u);
    const uint32_t bp = b0 + (pass == 1 ? b_part : 0u);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const uint64_t ad = make_desc_sw128(ap + 32 * ks);
      const uint64_t bd = make_desc_sw128(bp + 32 * ks);
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
          "l"(ad), "l"(bd), "r"(idesc), "r"(acc_in));
      acc_in = 1;
    }
  }
}

// One work item as every role of the CTA sees it.
struct TcItem {
  const float2* pb;  // this particle's spectra from the group's first psi
  int e0, a0, nd, psi0, g_psi;
};

__device__ __forceinline__ TcItem tc_item(const TcParams& P, int wi, int n, int H, int psi_group) {
  const int n_groups = (P.n_psi + psi_group - 1) / psi_group;
  const int b = P.work[2 * wi], tile = P.work[2 * wi + 1] / n_groups;
  TcItem it;
  it.psi0 = (P.work[2 * wi + 1] - tile * n_groups) * psi_group;
  it.g_psi = min(psi_group, P.n_psi - it.psi0);
  it.e0 = P.local_ptr[b];
  const int d = P.local_ptr[b + 1] - it.e0;
  it.a0 = tile * P.dpt;
  it.nd = min(P.dpt, d - it.a0);
  it.pb = P.stack + ((size_t)b * P.n_psi + it.psi0) * n * H;
  return it;
}

// byte offset of 16-byte chunk c of row j in a 128-byte-swizzled K-major tile
__device__ __forceinline__ uint32_t sw128(int j, int c) {
  return (uint32_t)(j * 128 + ((c ^ (j & 7)) << 4));
}

// Row stride (complex entries) of the table of w^{r y}: n plus two, so the
// rows of consecutive crop rows start 16 bytes apart and the eight 16-byte
// loads of a quarter warp fall on distinct banks.
__host__ __device__ constexpr int tc_twy_ld(int n) { return n + 2; }

// B for one K step: one task per (psi, crop row, 8-row block). The eight
// rows of the particle column times their twiddles w^{r y} (from a table in
// shared memory, row yi for y = yi - C/2), times the operand and column
// scale; Re U and Im U go to the psi's Re-Z and Im-Z rows (Re U, -Im U on
// the imaginary half of the Re-Z row). The products of a task are
// independent of one another (a twiddle recurrence along the rows made each
// depend on the previous one; the table measured 1-2% faster and is exact to
// the table's rounding).
template <int C, int N, bool BF>
__device__ __forceinline__ void build_b_step(unsigned char* stB, uint32_t b_part, const float2* sp,
                                             const float2* s_twy, float scale, int qq, int g_psi, bool split,
                                             int bt) {
  constexpr int n = N, kPS = tc_psi_stride(C), LD = tc_twy_ld(N);
  const int tasks = g_psi * C * 4;
  for (int t = bt; t < tasks; t += kTcBuilders) {
    const int yi = t % C, rc = (t / C) & 3, s = t / (4 * C);
    const int r0 = qq * 32 + rc * 8;
    const float4* pp = reinterpret_cast<const float4*>(sp + s * n + r0);
    const float4* ww = reinterpret_cast<const float4*>(s_twy + yi * LD + r0);
    uint32_t hr[4], lr[4], hi_[4], li_[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 p2 = pp[i], w2 = ww[i];
      const float2 u0 = cscale(cmul(make_float2(p2.x, p2.y), make_float2(w2.x, w2.y)), scale);
      const float2 u1 = cscale(cmul(make_float2(p2.z, p2.w), make_float2(w2.z, w2.w)), scale);
      split2<BF>(u0.x, u1.x, hr[i], lr[i]);
      split2<BF>(u0.y, u1.y, hi_[i], li_[i]);
    }
    const int jr = s * kPS + 4 * (yi >> 1) + (yi & 1), ji = jr + 2;
    const uint4 hre = make_uint4(hr[0], hr[1], hr[2], hr[3]), him = make_uint4(hi_[0], hi_[1], hi_[2], hi_[3]);
    *reinterpret_cast<uint4*>(stB + sw128(jr, rc)) = hre;
    *reinterpret_cast<uint4*>(stB + sw128(ji, 4 + rc)) = hre;
    *reinterpret_cast<uint4*>(stB + sw128(ji, rc)) = him;
    *reinterpret_cast<uint4*>(stB + sw128(jr, 4 + rc)) = neg8(him);
    if (split) {
      const uint4 lre = make_uint4(lr[0], lr[1], lr[2], lr[3]), lim = make_uint4(li_[0], li_[1], li_[2], li_[3]);
      *reinterpret_cast<uint4*>(stB + b_part + sw128(jr, rc)) = lre;
      *reinterpret_cast<uint4*>(stB + b_part + sw128(ji, 4 + rc)) = lre;
      *reinterpret_cast<uint4*>(stB + b_part + sw128(ji, rc)) = lim;
      *reinterpret_cast<uint4*>(stB + b_part + sw128(jr, 4 + rc)) = neg8(lim);
    }
  }
}

template <int C, int N, bool BF>
__global__ void __launch_bounds__(kTcThreads, 1) correlate_tc(TcParams P) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  static_assert(C % 2 == 0 && C <= 14, "even crop up to 14");
  static_assert(kTcThreads == 32 * (kTcEpiWarp0 + kTcEpiWarps), "warp roles");
  static_assert(kTcEpiWarps == 4 * 3, "three psi angles of four TMEM lane quarters");
  // TMEM: two accumulators of kN columns, then (C - RR) crop rows of C
  // columns for each psi of the group (warps of a psi past the group never
  // touch TMEM); a psi's accumulator columns lie inside the accumulator
  static_assert(2 * tc_n(C) + tc_psi_group(C) * (C - tc_reg_rows<C>()) * C <= kTcTmemCols, "TMEM columns");
  static_assert(tc_psi_group(C) * tc_psi_stride(C) <= tc_n(C), "psi rows of the accumulator");
  constexpr int kN = tc_n(C);
  constexpr int kPS = tc_psi_stride(C);
  constexpr int NQ = N / 32;               // K steps per column: 32 rows r (64 K) each
  constexpr int n = N, H = N / 2 + 1;
  constexpr int TWE = tc_tw_entries(C);
  constexpr uint32_t a_part = kTcM * 128;  // bytes of A (hi or lo) per step: 128 rows x 128 B
  constexpr uint32_t b_part = kN * 128;    // bytes of B (hi or lo) per step
  static_assert(a_part % 1024 == 0 && b_part % 1024 == 0, "stages keep the 1024-byte swizzle alignment");
  const int parts = P.split ? 2 : 1;
  const int SA = P.sa, SB = P.sb;
  const uint32_t a_bytes = parts * a_part, b_bytes = parts * b_part;
  const int n_cand = P.n_cand;
  const int nc8 = (n_cand + 7) & ~7;       // rows per direction in a tile
  unsigned char* ring_a = smem_raw;                  // [SA][part][128 rows][128 B]
  unsigned char* ring_b = smem_raw + SA * a_bytes;   // [SB][part][kN rows][128 B]
  float2* s_p = reinterpret_cast<float2*>(ring_b + SB * b_bytes);  // [3][kTcPsi][n] particle columns
  float2* s_twy = s_p + 3 * kTcPsi * n;                        // [C][tc_twy_ld(n)] w^{r y}
  float* s_twall = reinterpret_cast<float*>(s_twy + C * tc_twy_ld(n));  // [H][TWE] column tables
  float* s_psc = s_twall + H * TWE;                           // [H] particle-side scale per column
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_psc + ((H + 1) & ~1));
  uint64_t* bar_afull = s_bar;                    // [SA] A bytes landed (copy warp's expect_tx)
  uint64_t* bar_aempty = s_bar + kTcMaxSA;        // [SA] the MMAs reading the A stage are done
  uint64_t* bar_bfull = s_bar + 2 * kTcMaxSA;     // [SB] every builder warp wrote B
  uint64_t* bar_bempty = bar_bfull + kTcMaxSB;    // [SB] the MMAs reading the B stage are done
  uint64_t* bar_tfull = bar_bempty + kTcMaxSB;    // [2] a column's accumulator is final
  uint64_t* bar_tempty = bar_tfull + 2;           // [2] every stage-2 warp read its accumulator
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bar_tempty + 2);
  int* s_fail = reinterpret_cast<int*>(s_taddr + 1);
  uint32_t* s_mma_steps = reinterpret_cast<uint32_t*>(s_fail + 1);   // K steps whose MMAs were committed
  uint32_t* s_copy_steps = s_mma_steps + 1;                           // K steps whose A copies were issued

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int t = tid; t < C * n; t += blockDim.x) {
    const int yi = t / n, r = t - yi * n, y = yi - C / 2;
    s_twy[yi * tc_twy_ld(n) + r] = P.tw_row[((r * y) % n + n) % n];
  }
  for (int t = tid; t < H * TWE; t += blockDim.x) {
    const int c = t / TWE;
    const float ts = P.t_scale ? P.t_scale[c] : 1.0f, ps = P.p_scale ? P.p_scale[c] : 1.0f;
    s_twall[t] = tw_entry<C>(P.tw_col, c, t % TWE, 1.0f / (kTcScale * kTcScale * ts * ps));
  }
  for (int t = tid; t < H; t += blockDim.x) s_psc[t] = kTcScale * (P.p_scale ? P.p_scale[t] : 1.0f);
  for (uint32_t t = tid; t < (SA * a_bytes + SB * b_bytes) / 16; t += blockDim.x)
    reinterpret_cast<uint4*>(smem_raw)[t] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    for (int i = 0; i < SA; ++i) {
      mbar_init(bar_afull + i, 1);
      mbar_init(bar_aempty + i, 1);
    }
    for (int i = 0; i < SB; ++i) {
      mbar_init(bar_bfull + i, kTcBuildWarps);
      mbar_init(bar_bempty + i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar_tfull + i, 1);
      mbar_init(bar_tempty + i, kTcEpiWarps);
    }
    *s_fail = 0;
    *s_mma_steps = 0;
    *s_copy_steps = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_taddr)),
                 "r"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t taddr = *s_taddr;
  const unsigned limit = P.wait_limit;

  // bounded wait that gives up at once after any failure in the CTA
  auto wait = [&](uint64_t* bar, uint32_t parity) -> bool {
    if (*reinterpret_cast<volatile int*>(s_fail) != 0) return false;
    const bool r = mbar_wait(bar, parity, limit);
    if (!r) *reinterpret_cast<volatile int*>(s_fail) = 1;
    return r;
  };

  // Ring positions: every role walks the same K steps g = 0, 1, ...; step g
  // uses A stage g % SA and B stage g % SB, in use number g / SA (g / SB).
  // Consumers wait for the full barrier's phase (use & 1); producers of a
  // stage's next use wait for the empty barrier's previous phase.
  if (warp == 0) {
    // ---------------- MMA issue (one lane)
    if (lane == 0) {
      uint32_t g = 0, tuse[2] = {0, 0}, pa = 0, pb = 0;
      int ia = 0, ib = 0;
      const uint32_t idesc = make_idesc(kTcM, kN, BF ? 1 : 0);
      bool ok = true;
      for (int wi = blockIdx.x; wi < P.n_work && ok; wi += gridDim.x) {
        for (int col = 0; col < H && ok; ++col) {
          const int tb = col & 1;
          for (int qq = 0; qq < NQ && ok; ++qq, ++g) {
            if (qq == 0 && tuse[tb] > 0) ok = wait(bar_tempty + tb, (tuse[tb] - 1) & 1u);
            ok = ok && wait(bar_bfull + ib, pb) && wait(bar_afull + ia, pa);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a0s = smem_u32(ring_a + ia * a_bytes), b0s = smem_u32(ring_b + ib * b_bytes);
            issue_mma_step(taddr + (uint32_t)(tb * kN), a0s, b0s, a_part, b_part, idesc, P.split ? 3 : 1, qq > 0);
            mma_commit(bar_aempty + ia);
            mma_commit(bar_bempty + ib);
            *s_mma_steps = g + 1;
            if (qq == NQ - 1) {
              mma_commit(bar_tfull + tb);
              ++tuse[tb];
            }
            if (++ia == SA) { ia = 0; pa ^= 1u; }
            if (++ib == SB) { ib = 0; pb ^= 1u; }
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- A: one bulk copy of n_cand 128-byte rows per (part, direction) and step,
    // and an L2 prefetch of each direction's rows two columns ahead
    const uint32_t bytes = (uint32_t)n_cand * 128;
    uint32_t g = 0, pa = 0;
    int ia = 0;
    int zeroed[kTcMaxSA];  // rows [zeroed[s], 128) of A stage s read as zero
#pragma unroll
    for (int s = 0; s < kTcMaxSA; ++s) zeroed[s] = 0;
    bool ok = true;
    for (int wi = blockIdx.x; wi < P.n_work && ok; wi += gridDim.x) {
      const TcItem it = tc_item(P, wi, n, H, tc_psi_group(C));
      const int used = it.nd * nc8;
      int slot = 0;
      if (lane < parts * it.nd) slot = P.local_idx[it.e0 + it.a0 + lane % it.nd];
      const unsigned char* bank = static_cast<const unsigned char*>(P.tbank);
      for (int col = 0; col < H && ok; ++col) {
        if (col + 2 < H) {
          // the parts of every (direction, K step) of column col + 2
          for (int t = lane; t < it.nd * NQ; t += 32) {
            const int d = t / NQ, q = t - d * NQ;
            const int sl = P.local_idx[it.e0 + it.a0 + d];
            const unsigned char* src = bank + ((((size_t)sl * H + col + 2) * NQ + q) * 2) * (size_t)bytes;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(parts * bytes) : "memory");
          }
        }
        for (int qq = 0; qq < NQ && ok; ++qq, ++g) {
          unsigned char* stA = ring_a + ia * a_bytes;
          if (g >= (uint32_t)SA) {
            bool w = true;
            if (lane == 0) w = wait(bar_aempty + ia, pa ^ 1u);
            ok = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
            if (!ok) break;
          }
#pragma unroll
          for (int s = 0; s < kTcMaxSA; ++s) {
            if (s == ia && used < zeroed[s]) {
              // rows this tile leaves empty must read as zero
              const int span = zeroed[s] - used;
              for (int t = lane; t < parts * span * 8; t += 32) {
                const int row = used + (t >> 3) % span, part = (t >> 3) / span;
                *reinterpret_cast<uint4*>(stA + part * a_part + row * 128 + (t & 7) * 16) =
                    make_uint4(0, 0, 0, 0);
              }
              asm volatile("fence.proxy.async.shared::cta;");
              __syncwarp();
            }
            if (s == ia) zeroed[s] = used;
          }
          if (lane == 0) mbar_expect_tx(bar_afull + ia, (uint32_t)(parts * it.nd) * bytes);
          __syncwarp();
          if (lane < parts * it.nd) {
            const int part = lane / it.nd, dl = lane - part * it.nd;
            const unsigned char* src = bank + ((((size_t)slot * H + col) * NQ + qq) * 2 + part) * (size_t)bytes;
            bulk_copy(stA + part * a_part + (uint32_t)dl * nc8 * 128, src, bytes, bar_afull + ia);
          }
          if (lane == 0) *s_copy_steps = g + 1;
          if (++ia == SA) { ia = 0; pa ^= 1u; }
        }
      }
    }
  } else if (warp < kTcEpiWarp0) {
    // ---------------- B: U_{s,y}(r) = P_s(r, col) w^{r y}, scaled and split, per K step.
    // The builder warps always run the same sequence of named barriers (no
    // early exit): after a failure they only skip the work.
    const int bt = tid - 32 * kTcBuildWarp0;
    uint32_t g = 0, pb = 0;
    int ib = 0;
    bool ok = true;
    for (int wi = blockIdx.x; wi < P.n_work; wi += gridDim.x) {
      const TcItem it = tc_item(P, wi, n, H, tc_psi_group(C));
      const int g_psi = it.g_psi;
      // columns 0 and 1 of this particle; later columns arrive by cp.async two
      // columns ahead (one group per column and thread)
      asm volatile("bar.sync 1, %0;" ::"n"(kTcBuilders) : "memory");  // every builder left the previous item
      for (int t = bt; t < g_psi * n; t += kTcBuilders) {
        const int s = t / n, r = t - s * n;
        const float2* pcol = it.pb + ((size_t)s * n + r) * H;
        s_p[t] = __ldg(pcol);
        s_p[kTcPsi * n + t] = __ldg(pcol + 1);
      }
      for (int col = 0; col < H; ++col) {
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        asm volatile("bar.sync 1, %0;" ::"n"(kTcBuilders) : "memory");  // column col visible; col-1 done
        if (col + 2 < H) {
          for (int t = bt; t < g_psi * n; t += kTcBuilders) {
            const int s = t / n, r = t - s * n;
            cp_async8(s_p + ((col + 2) % 3) * kTcPsi * n + t, it.pb + ((size_t)s * n + r) * H + col + 2);
          }
        }
        asm volatile("cp.async.commit_group;");
        const float2* sp = s_p + (col % 3) * kTcPsi * n;
        const float scale = s_psc[col];
        for (int qq = 0; qq < NQ; ++qq, ++g) {
          unsigned char* stB = ring_b + ib * b_bytes;
          if (g >= (uint32_t)SB) ok = wait(bar_bempty + ib, pb ^ 1u) && ok;
          if (ok) build_b_step<C, N, BF>(stB, b_part, sp, s_twy, scale, qq, g_psi, P.split != 0, bt);
          asm volatile("fence.proxy.async.shared::cta;");
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_bfull + ib);
          if (++ib == SB) { ib = 0; pb ^= 1u; }
        }
      }
      asm volatile("cp.async.wait_all;" ::: "memory");
    }
  } else {
    // ---------------- stage 2 and the first maximum per (row, psi)
    constexpr int RR = tc_reg_rows<C>();  // crop rows in registers; rows [RR, C) in TMEM
    const int q4 = warp & 3, my_psi = (warp - kTcEpiWarp0) >> 2;
    // warps of a psi index past the tile's psi group (the third at crop 14)
    // own no TMEM rows and never touch TMEM
    const bool psi_ok = my_psi < tc_psi_group(C);
    const int my_row = 32 * q4 + lane;
    const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
    const uint32_t ta_z = taddr + lane_off + (uint32_t)(my_psi * kPS);
    const uint32_t ta_acc = taddr + lane_off + (uint32_t)(2 * kN + my_psi * (C - RR) * C);
    uint32_t tuse[2] = {0, 0};
    bool ok = true;
    for (int wi = blockIdx.x; wi < P.n_work && ok; wi += gridDim.x) {
      const bool active = my_psi < tc_item(P, wi, n, H, tc_psi_group(C)).g_psi;  // warp-uniform
      float acc[RR][C];  // [crop row][slot]
#pragma unroll
      for (int y = 0; y < RR; ++y)
#pragma unroll
        for (int j = 0; j < C; ++j) acc[y][j] = 0.f;
      if constexpr (RR < C) {
        if (psi_ok) {
          float z[C];
#pragma unroll
          for (int j = 0; j < C; ++j) z[j] = 0.f;
#pragma unroll
          for (int y = RR; y < C; ++y) tmem_st_row<C>(z, ta_acc + (uint32_t)((y - RR) * C));
          asm volatile("tcgen05.wait::st.sync.aligned;");
        }
      }
      for (int col = 0; col < H && ok; ++col) {
        const int tb = col & 1;
        ok = wait(bar_tfull + tb, tuse[tb] & 1u);
        ++tuse[tb];
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (active) {
          const uint32_t e = smem_u32(s_twall + col * TWE);
          const uint32_t tz = ta_z + (uint32_t)(tb * kN);
#pragma unroll
          for (int yp = 0; yp < C / 2; ++yp) {
            uint32_t v[4];  // Re Z(2yp), Re Z(2yp+1), Im Z(2yp), Im Z(2yp+1)
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                         : "r"(tz + 4 * yp));
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int hy = 0; hy < 2; ++hy) {
              const int y = 2 * yp + hy;
              const float zr = __uint_as_float(v[hy]), zi = __uint_as_float(v[2 + hy]);
              if (y < RR) {
                stage2_row<C>(acc[y < RR ? y : 0], zr, zi, e);
              } else {
                float a[C];
                tmem_ld_row<C>(a, ta_acc + (uint32_t)((y - RR) * C));
                stage2_row<C>(a, zr, zi, e);
                tmem_st_row<C>(a, ta_acc + (uint32_t)((y - RR) * C));
              }
            }
          }
          asm volatile("tcgen05.wait::st.sync.aligned;");
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_tempty + tb);
      }
      if (!ok) break;
      // the first maximum, row-major over (y, x): register rows, then TMEM rows
      float best = -INFINITY;
      int bi = 0;
#pragma unroll
      for (int y = 0; y < RR; ++y) {
#pragma unroll
        for (int x = 0; x < C; ++x) {
          const float v = raw_at<C>(acc[y], x);
          if (v > best) {
            best = v;
            bi = y * C + x;
          }
        }
      }
      if (psi_ok) {
#pragma unroll
        for (int y = RR; y < C; ++y) {
          float a[C];
          tmem_ld_row<C>(a, ta_acc + (uint32_t)((y - RR) * C));
#pragma unroll
          for (int x = 0; x < C; ++x) {
            const float v = raw_at<C>(a, x);
            if (v > best) {
              best = v;
              bi = y * C + x;
            }
          }
        }
      }
      const TcItem it = tc_item(P, wi, n, H, tc_psi_group(C));
      const int dl = my_row / nc8, cand = my_row - dl * nc8;
      if (active && dl < it.nd && cand < n_cand) {
        const size_t o = (size_t)cand * P.nnz * P.n_psi + (size_t)(it.e0 + it.a0 + dl) * P.n_psi + it.psi0 + my_psi;
        P.out_score[o] = best * 1024.0f;
        P.out_y[o] = bi / C;
        P.out_x[o] = bi % C;
      }
    }
  }
  // Every role has left its loop. After a failure, the bulk copies and the
  // MMAs this CTA issued get a last bounded chance (the default bound) to
  // finish before the CTA frees its TMEM and exits: the latest use of each
  // A stage is among the last SA steps issued (every MMA commit also covers
  // the MMAs before it, so the A ring's barriers cover the B ring's readers).
  __syncthreads();
  if (*reinterpret_cast<volatile int*>(s_fail) != 0) {
    if (tid == 0) {
      if (P.status != nullptr) atomicExch(P.status, 1);
      const uint32_t gm = *s_mma_steps, ga = *s_copy_steps, sa = (uint32_t)SA;
      for (uint32_t g = gm > sa ? gm - sa : 0; g < gm; ++g)
        mbar_wait(bar_aempty + g % sa, (g / sa) & 1u, kWaitLimit);
      for (uint32_t g = ga > sa ? ga - sa : 0; g < ga; ++g)
        mbar_wait(bar_afull + g % sa, (g / sa) & 1u, kWaitLimit);
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTcTmemCols));
  }
}

// Operand copy of template banks for the tensor-core kernel:
// out[slot][col][step][part][cand][128 B]; part 0 hi, part 1 lo (split
// forms only read part 1). Step q covers rows r in [32q, 32q + 32): logical
// 16-byte chunk c < 4 holds Re T of rows 32q + 8c.., chunk 4 + c holds Im T
// of the same rows, scaled by 2^13 times the column's scale; chunk c is
// stored at position c ^ (cand & 7) (the 128-byte swizzle of the
// shared-memory tile, whose direction blocks start on multiples of 8 rows).
// One block per (slot, candidate); every candidate writes whole 128-byte
// rows. The lo halves are written for the split forms only (the single
// forms never read them). A value that leaves the operand type's range sets
// *status to 2.
__host__ __device__ inline int bank_fp16_ld(int n) { return n + n / 8 + 1; }

template <bool BF>
__global__ void bank_to_operands(const float2* __restrict__ bank, long long bank_stride, int n, int n_cand,
                                 int cb, const float* __restrict__ t_scale, unsigned char* __restrict__ out,
                                 int split, int* status) {
  // [cb][ld]: columns [c0, c0 + cb) of the template, column-major with a
  // spare slot after every 8 rows, so the 16 row blocks a warp reads at once
  // fall on distinct banks
  extern __shared__ float2 s_t[];
  const int H = n / 2 + 1, nq = n / 32, ld = bank_fp16_ld(n);
  const int slot = blockIdx.x, cand = blockIdx.y;
  const float2* src = bank + (size_t)cand * (size_t)bank_stride + (size_t)slot * n * H;
  bool bad = false;
  for (int c0 = 0; c0 < H; c0 += cb) {
    const int w = min(cb, H - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < n * w; t += blockDim.x) {
      const int r = t / w, c = t - r * w;
      s_t[c * ld + r + (r >> 3)] = src[(size_t)r * H + c0 + c];
    }
    __syncthreads();
    // one task per (col, step, chunk): 8 consecutive k -> hi and lo 16-byte chunks
    for (int t = threadIdx.x; t < w * nq * 8; t += blockDim.x) {
      const int c = t & 7, qq = (t >> 3) % nq, cl = t / (8 * nq), col = c0 + cl;
      const bool imag = c >= 4;
      const int r0 = qq * 32 + (c & 3) * 8;
      const float2* sc = s_t + cl * ld + r0 + (r0 >> 3);
      const float scale = kTcScale * (t_scale ? t_scale[col] : 1.0f);
      uint32_t h[4], l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float2 z0 = sc[2 * i], z1 = sc[2 * i + 1];
        const float a = (imag ? z0.y : z0.x) * scale, b = (imag ? z1.y : z1.x) * scale;
        bad |= !(fabsf(a) <= (BF ? 3.0e38f : 65504.0f)) || !(fabsf(b) <= (BF ? 3.0e38f : 65504.0f));
        split2<BF>(a, b, h[i], l[i]);
      }
      const size_t row = (((size_t)slot * H + col) * nq + qq) * 2;  // part 0 row block
      const int pos = c ^ (cand & 7);
      *reinterpret_cast<uint4*>(out + ((row * n_cand + cand) * 8 + pos) * 16) = make_uint4(h[0], h[1], h[2], h[3]);
      if (split)
        *reinterpret_cast<uint4*>(out + (((row + 1) * n_cand + cand) * 8 + pos) * 16) =
            make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
  if (bad && status != nullptr) atomicExch(status, 2);
}

template <int C, int N, bool BF>
cudaError_t launch_tc_cnb(const TcParams& P, size_t smem, int grid, cudaStream_t st) {
  static size_t set_smem = 0;
  if (set_smem < smem) {
    cudaError_t e =
        cudaFuncSetAttribute(correlate_tc<C, N, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    set_smem = smem;
  }
  correlate_tc<C, N, BF><<<grid, kTcThreads, smem, st>>>(P);
  return cudaGetLastError();
}

template <int C, int N>
cudaError_t launch_tc_cn(const TcParams& P, size_t smem, int grid, cudaStream_t st) {
  return P.bf16 ? launch_tc_cnb<C, N, true>(P, smem, grid, st) : launch_tc_cnb<C, N, false>(P, smem, grid, st);
}

template <int C>
cudaError_t launch_tc_c(const TcParams& P, size_t smem, int grid, cudaStream_t st) {
  switch (P.n) {
    case 32: return launch_tc_cn<C, 32>(P, smem, grid, st);
    case 64: return launch_tc_cn<C, 64>(P, smem, grid, st);
    case 96: return launch_tc_cn<C, 96>(P, smem, grid, st);
    case 128: return launch_tc_cn<C, 128>(P, smem, grid, st);
    case 192: return launch_tc_cn<C, 192>(P, smem, grid, st);
    case 256:
      if constexpr (C >= 10) return launch_tc_cn<C, 256>(P, smem, grid, st);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

int correlate_tc_max_psi() { return kTcPsi; }
int correlate_tc_max_n() { return kTcMaxN; }
int correlate_tc_max_cand() { return kTcMaxCand; }
unsigned correlate_tc_default_wait() { return kWaitLimit; }

// Shared memory after the rings: particle columns, tables, barriers, TMEM
// address and status words.
static size_t tc_tail_bytes(int n, int crop) {
  const int H = n / 2 + 1;
  return 3 * (size_t)kTcPsi * n * sizeof(float2) + (size_t)crop * tc_twy_ld(n) * sizeof(float2) +
         (size_t)H * tc_tw_entries(crop) * sizeof(float) + (size_t)((H + 1) & ~1) * sizeof(float) +
         (2 * kTcMaxSA + 2 * kTcMaxSB + 4) * 8 + 16;
}
static size_t tc_a_bytes(int split) { return (split ? 2 : 1) * (size_t)kTcM * 128; }
static size_t tc_b_bytes(int crop, int split) { return (split ? 2 : 1) * (size_t)tc_n(crop) * 128; }

// Ring depths of a launch: the requested ones (0: the default, A four deep
// and B two deep) within their limits, A reduced to what the shared memory
// holds. Deeper A rings did not help on GB300: the shared memory they take
// comes out of the L1 cache that holds the particle rows the B build
// gathers (at box 128 a particle's three psi rows are 48 KB of lines).
// Returns false when not even two A stages fit.
bool correlate_tc_rings(int n, int crop, int split, int want_sa, int want_sb, int* sa, int* sb) {
  const long long avail = (long long)kTcSmemMax - (long long)tc_tail_bytes(n, crop);
  const long long a = (long long)tc_a_bytes(split), b = (long long)tc_b_bytes(crop, split);
  const int B = want_sb > 0 ? std::min(want_sb, kTcMaxSB) : 2;
  const int A = (int)std::min<long long>(want_sa > 0 ? std::min(want_sa, kTcMaxSA) : 4, (avail - B * b) / a);
  if (A < 2) return false;
  *sa = A;
  *sb = B;
  return true;
}

size_t correlate_tc_smem_bytes(int n, int crop, int split, int sa, int sb) {
  return sa * tc_a_bytes(split) + sb * tc_b_bytes(crop, split) + tc_tail_bytes(n, crop);
}

// bytes of the operand copy of one candidate's bank: hi and lo halves
long long correlate_tc_bank_halves(int n_slot, int n) {
  return (long long)n_slot * (n / 2 + 1) * 2 * (2LL * n);
}

// directions per tile for a launch of n_cand candidates (rows per direction
// rounded up to 8, the swizzle atom)
int correlate_tc_dirs_per_tile(int n_cand) {
  return n_cand > 0 ? kTcM / ((std::min(n_cand, kTcMaxCand) + 7) & ~7) : 0;
}

// Work list (particle, tile * n_groups + psi group) for the tensor-core
// kernel, sorted by the tile's direction slots (lexicographically, then
// particle), so that tiles with the same directions run one after another
// and CTAs running at the same time read the same template columns from L2
// (at box 128 with 5,000 particles and 64 candidates: 14,831 tiles of 2,715
// distinct direction pairs). A tile holds 128 / n_cand whole directions
// (n_cand <= 128). Host arrays; returns the item count.
int correlate_tc_plan(const int* local_ptr, const int* local_idx, int n_particles, int n_cand, int n_psi, int crop,
                      int* work, int max_work) {
  struct Item { int e, len, b, tile; };
  const int pg = tc_psi_group(crop);
  const int n_groups = (n_psi + pg - 1) / pg;
  const int dpt = correlate_tc_dirs_per_tile(n_cand);
  std::vector<Item> items;
  for (int b = 0; b < n_particles; ++b) {
    const int e0 = local_ptr[b], d = local_ptr[b + 1] - e0;
    const int tiles = (d + dpt - 1) / dpt;
    for (int t = 0; t < tiles; ++t)
      for (int g = 0; g < n_groups; ++g)
        items.push_back({e0 + t * dpt, std::min(dpt, d - t * dpt), b, t * n_groups + g});
  }
  std::stable_sort(items.begin(), items.end(), [local_idx](const Item& x, const Item& y) {
    return std::lexicographical_compare(local_idx + x.e, local_idx + x.e + x.len, local_idx + y.e,
                                        local_idx + y.e + y.len);
  });
  const int count = (int)items.size();
  if (work != nullptr) {
    for (int i = 0; i < count && i < max_work; ++i) {
      work[2 * i] = items[i].b;
      work[2 * i + 1] = items[i].tile;
    }
  }
  return count;
}

cudaError_t launch_bank_to_operands(cudaStream_t st, const float2* bank, long long bank_stride, int n_cand,
                                    int n_slot, int n, int bf16, int split, const float* t_scale, void* out,
                                    int* status) {
  if (n_cand <= 0 || n_slot <= 0) return cudaSuccess;
  // columns per pass of a block: 16 (18.6 KB of shared memory at n = 128)
  // keeps about ten blocks resident per SM, so loads of some blocks overlap
  // the conversion and stores of others (all 65 columns in one pass, 75 KB,
  // ran the copy at 2.6 TB/s; 16 columns took 1.1 ms less per 64-candidate
  // bank at box 128)
  const int cb = std::min(n / 2 + 1, 16);
  const size_t smem = (size_t)bank_fp16_ld(n) * cb * sizeof(float2);
  static size_t set_smem[2] = {0, 0};
  const int k = bf16 ? 1 : 0;
  if (set_smem[k] < smem) {
    cudaError_t e = bf16 ? cudaFuncSetAttribute(bank_to_operands<true>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                         : cudaFuncSetAttribute(bank_to_operands<false>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    set_smem[k] = smem;
  }
  if (bf16)
    bank_to_operands<true><<<dim3(n_slot, n_cand), 256, smem, st>>>(bank, bank_stride, n, n_cand, cb, t_scale,
                                                                     (unsigned char*)out, split, status);
  else
    bank_to_operands<false><<<dim3(n_slot, n_cand), 256, smem, st>>>(bank, bank_stride, n, n_cand, cb, t_scale,
                                                                      (unsigned char*)out, split, status);
  return cudaGetLastError();
}

cudaError_t launch_correlate_tc(cudaStream_t st, const void* tbank, int n_cand, const float2* stack,
                                const int* local_ptr, const int* local_idx, const int* work, int n_work, int n_psi,
                                int n, int crop, int nnz, int split, int bf16, const float* t_scale,
                                const float* p_scale, unsigned wait_limit, const float2* tw_row,
                                const float2* tw_col, float* out_score, int* out_y, int* out_x, int* status,
                                int grid, int want_sa, int want_sb) {
  if (n_work <= 0 || n_cand <= 0) return cudaSuccess;
  if (n_cand > kTcMaxCand) return cudaErrorInvalidValue;
  int sa = 0, sb = 0;
  if (!correlate_tc_rings(n, crop, split, want_sa, want_sb, &sa, &sb)) return cudaErrorInvalidValue;
  TcParams P;
  P.tbank = tbank;
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
  P.bf16 = bf16 ? 1 : 0;
  P.dpt = correlate_tc_dirs_per_tile(n_cand);
  P.tw_row = tw_row;
  P.tw_col = tw_col;
  P.t_scale = t_scale;
  P.p_scale = p_scale;
  P.wait_limit = wait_limit ? wait_limit : kWaitLimit;
  P.out_score = out_score;
  P.out_y = out_y;
  P.out_x = out_x;
  P.status = status;
  P.sa = sa;
  P.sb = sb;

  const size_t smem = correlate_tc_smem_bytes(n, crop, split, sa, sb);
  switch (crop) {
    case 2: return launch_tc_c<2>(P, smem, grid, st);
    case 4: return launch_tc_c<4>(P, smem, grid, st);
    case 6: return launch_tc_c<6>(P, smem, grid, st);
    case 8: return launch_tc_c<8>(P, smem, grid, st);
    case 10: return launch_tc_c<10>(P, smem, grid, st);
    case 12: return launch_tc_c<12>(P, smem, grid, st);
    case 14: return launch_tc_c<14>(P, smem, grid, st);
    default: return cudaErrorInvalidValue;
  }
}
