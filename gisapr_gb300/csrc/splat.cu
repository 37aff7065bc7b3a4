// Gaussian atom splat (pdb2mrc density) for sm_103a.
//
// Two launches:
//   1. atoms_prepare: one thread per atom. Optional rigid-body pose in FP64
//      ((c - pivot) @ R + pivot + t), the PDB 8.3 write/reread, the voxel
//      position f32(f64(q)/apix + box/2) and the clipped integer bounds
//      (pdb_text.py:123-142, ZL pdb_text.py:33-58, pdb2mrc_gpu_ver_fp32_v3.py:
//      71-87).
//   2. splat_bricks: one CTA per 16^3 brick of the box. Each thread owns one
//      (x, y) column of 16 voxels in registers and walks the atoms in input
//      order, so every voxel sums its contributions in the reference's atom
//      order with no atomics: the result is deterministic, and a cached
//      fixed-context brick is read once and written once (no clone pass).
//      The epilogue optionally writes the sinc^2-weighted value into the
//      zero-padded, fftshifted (2N)^3 input of the volume FFT (v606:837-853,
//      1063-1072), so the padded volume is never materialised separately.
//
// Per voxel the arithmetic follows the reference's float32/float64 mix
// (pdb2mrc:88-95): r = sqrtf((dx*dx + dy*dy) + dz*dz) with every product and
// sum rounded to float; exponent = f32(-r * rp) and value = f32(Z*kn *
// expf(exponent)) where rp and Z*kn are doubles. The float64 products are
// formed in float32 pairs (hi + lo) with an exact product error term, which
// gives the same float result as the double product except at exact ties.
#include <climits>

#include "common.cuh"

namespace {

constexpr int kBrick = 16;

struct AtomRec {
  float px, py, pz;   // voxel-space position (float32)
  int lx, ly, lz;     // clipped lower bounds (inclusive)
  int ux, uy, uz;     // clipped upper bounds (exclusive)
  float zk_hi, zk_lo; // Z*kn as a float pair (0 => atom skipped)
  int pad;
};
static_assert(sizeof(AtomRec) == 48, "AtomRec layout");

__device__ __forceinline__ int round_away_f64(double v) {
  double a = floor(fabs(v) + 0.5);
  return (int)(v < 0.0 ? -a : a);
}

// Round v*1000 to the nearest integer, ties to even, using the exact
// product v*1000 = hi + lo (fma residual). This is what Python's "%8.3f"
// does with the exact binary value of v.
__device__ __forceinline__ double pdb_8_3(double v) {
  double hi = v * 1000.0;
  double lo = fma(v, 1000.0, -hi);
  double f = floor(hi);
  double d = (hi - f) - 0.5;  // exact for |hi| < 2^52
  d += lo;
  double r;
  if (d > 0.0) r = f + 1.0;
  else if (d < 0.0) r = f;
  else r = (fmod(f, 2.0) == 0.0) ? f : f + 1.0;
  // hi may itself sit on an integer with lo carrying the sign of the error.
  if (hi == f && lo < 0.0) {
    // exact value slightly below the integer hi: nearest is still hi unless
    // the distance reaches a half (impossible for |lo| < 0.5).
    r = f;
  }
  return r / 1000.0;
}

__global__ void atoms_prepare(const float* __restrict__ xyz, const float* __restrict__ numbers,
                              int n, int transform, const float* __restrict__ pivot,
                              const double* __restrict__ rot, const double* __restrict__ shift,
                              int box, int width, double apix, double kn,
                              AtomRec* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float c[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  float q[3];
  if (transform) {
    // (c - pivot) is float32, as numpy evaluates float32 arrays; the matrix
    // product and the additions are float64 (pdb_text.py:141).
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = (double)__fsub_rn(c[k], pivot[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double m = d[0] * rot[0 * 3 + k];
      m = fma(d[1], rot[1 * 3 + k], m);
      m = fma(d[2], rot[2 * 3 + k], m);
      double v = m + (double)pivot[k] + shift[k];
      q[k] = (float)pdb_8_3(v);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = c[k];
  }
  AtomRec r;
  float p[3];
  int lo[3], hi[3];
  bool inside = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[k] = (float)((double)q[k] / apix + (double)(box / 2));
    lo[k] = round_away_f64((double)__fsub_rn(p[k], (float)width));
    hi[k] = round_away_f64((double)__fadd_rn(p[k], (float)width));
    inside = inside && (lo[k] < box) && (hi[k] >= 0);
    lo[k] = max(lo[k], 0);
    hi[k] = min(hi[k], box - 1);
  }
  const float z = numbers[i];
  double zk = (double)z * kn;
  float zk_hi = (float)zk;
  float zk_lo = (float)(zk - (double)zk_hi);
  if (!inside || z == 0.0f || !(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) {
    zk_hi = 0.0f;
    zk_lo = 0.0f;
  }
  r.px = p[0]; r.py = p[1]; r.pz = p[2];
  r.lx = lo[0]; r.ly = lo[1]; r.lz = lo[2];
  r.ux = hi[0]; r.uy = hi[1]; r.uz = hi[2];
  r.zk_hi = zk_hi; r.zk_lo = zk_lo; r.pad = 0;
  out[i] = r;
}



__global__ void __launch_bounds__(256)
splat_bricks(const AtomRec* __restrict__ atoms, int n_atoms, const float* initial,
             float* out, float* __restrict__ padded, int box, float rp_hi,
             float rp_lo) {
  __shared__ AtomRec s_atoms[256];
  __shared__ int s_count;
  const int nbx = (box + kBrick - 1) / kBrick;
  const int bz = blockIdx.x / (nbx * nbx);
  const int by = (blockIdx.x / nbx) % nbx;
  const int bx = blockIdx.x % nbx;
  const int x = bx * kBrick + (threadIdx.x & 15);
  const int y = by * kBrick + (threadIdx.x >> 4);
  const int z0 = bz * kBrick;
  const bool col_ok = (x < box) && (y < box);
  const size_t plane = (size_t)box * box;

  float acc[kBrick];
#pragma unroll
  for (int k = 0; k < kBrick; ++k) {
    const int z = z0 + k;
    acc[k] = (initial != nullptr && col_ok && z < box) ? initial[(size_t)z * plane + (size_t)y * box + x]
                                                       : 0.0f;
  }
  const int bx0 = bx * kBrick, by0 = by * kBrick;
  const float fx = (float)x, fy = (float)y;
  for (int base = 0; base < n_atoms; base += 256) {
    const int ai = base + threadIdx.x;
    __syncthreads();
    if (threadIdx.x == 0) s_count = 0;
    bool hit = false;
    AtomRec r;
    if (ai < n_atoms) {
      r = atoms[ai];
      hit = (r.zk_hi != 0.0f || r.zk_lo != 0.0f) && r.ux > bx0 && r.lx < bx0 + kBrick &&
            r.uy > by0 && r.ly < by0 + kBrick && r.uz > z0 && r.lz < z0 + kBrick;
    }
    // Order-preserving compaction of the atoms that touch this brick.
    const unsigned mask = __ballot_sync(0xffffffffu, hit);
    __syncthreads();
    __shared__ int s_warp_base[8];
    if ((threadIdx.x & 31) == 0) s_warp_base[threadIdx.x >> 5] = __popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
      int run = 0;
      for (int w = 0; w < 8; ++w) {
        int c = s_warp_base[w];
        s_warp_base[w] = run;
        run += c;
      }
      s_count = run;
    }
    __syncthreads();
    if (hit) {
      const int pos = s_warp_base[threadIdx.x >> 5] + __popc(mask & ((1u << (threadIdx.x & 31)) - 1u));
      s_atoms[pos] = r;
    }
    __syncthreads();
    const int cnt = s_count;
    for (int t = 0; t < cnt; ++t) {
      const AtomRec a = s_atoms[t];
      if (!col_ok || x < a.lx || x >= a.ux || y < a.ly || y >= a.uy) continue;
      const float dx = __fsub_rn(fx, a.px), dy = __fsub_rn(fy, a.py);
      const float sxy = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
#pragma unroll
      for (int k = 0; k < kBrick; ++k) {
        const int z = z0 + k;
        if (z >= a.lz && z < a.uz) {
          const float dz = __fsub_rn((float)z, a.pz);
          const float rr = sqrtf(__fadd_rn(sxy, __fmul_rn(dz, dz)));
          // f32(r * rp) with rp = rp_hi + rp_lo
          const float ph = __fmul_rn(rr, rp_hi);
          const float pe = __fmaf_rn(rr, rp_hi, -ph);
          const float expo = -__fadd_rn(ph, __fmaf_rn(rr, rp_lo, pe));
          const float e = expf(expo);
          // f32(zk * e) with zk = zk_hi + zk_lo
          const float vh = __fmul_rn(a.zk_hi, e);
          const float ve = __fmaf_rn(a.zk_hi, e, -vh);
          const float v = __fadd_rn(vh, __fmaf_rn(a.zk_lo, e, ve));
          acc[k] = __fadd_rn(acc[k], v);
        }
      }
    }
  }
  if (!col_ok) return;
  const int m = 2 * box;
  const int half = box / 2;
  const float fyv = fftfreq_shifted_f32(y + half, m);
  const float fxv = fftfreq_shifted_f32(x + half, m);
  const float fy2 = __fmul_rn(fyv, fyv), fx2 = __fmul_rn(fxv, fxv);
  const size_t mm = (size_t)m * m;
  const int ys = (y + 3 * half) % m, xs = (x + 3 * half) % m;
#pragma unroll
  for (int k = 0; k < kBrick; ++k) {
    const int z = z0 + k;
    if (z >= box) break;
    if (out != nullptr) out[(size_t)z * plane + (size_t)y * box + x] = acc[k];
    if (padded != nullptr) {
      const float fzv = fftfreq_shifted_f32(z + half, m);
      const float w = sinc2_f32(__fmul_rn(fzv, fzv), fy2, fx2);
      const int zs = (z + 3 * half) % m;
      padded[(size_t)zs * mm + (size_t)ys * m + xs] = __fmul_rn(acc[k], w);
    }
  }
}

}  // namespace

// Host-side launchers (called from abi.cu).
cudaError_t launch_atoms_prepare(cudaStream_t st, const float* xyz, const float* numbers, int n,
                                 int transform, const float* pivot, const double* rot,
                                 const double* shift, int box, int width, double apix, double kn,
                                 void* atom_recs) {
  if (n <= 0) return cudaSuccess;
  atoms_prepare<<<(n + 255) / 256, 256, 0, st>>>(xyz, numbers, n, transform, pivot, rot, shift, box,
                                                  width, apix, kn, (AtomRec*)atom_recs);
  return cudaGetLastError();
}

size_t atom_record_bytes() { return sizeof(AtomRec); }

cudaError_t launch_splat_bricks(cudaStream_t st, const void* atom_recs, int n, const float* initial,
                                float* out, float* padded, int box, double rp) {
  const int nb = (box + kBrick - 1) / kBrick;
  const float rp_hi = (float)rp;
  const float rp_lo = (float)(rp - (double)rp_hi);
  splat_bricks<<<nb * nb * nb, 256, 0, st>>>((const AtomRec*)atom_recs, n, initial, out, padded, box,
                                             rp_hi, rp_lo);
  return cudaGetLastError();
}

namespace {
// Standalone sinc^2 / pad / fftshift of an existing box^3 density into the
// (2*box)^3 FFT input (the splat epilogue does the same for fresh densities).
__global__ void pad_sinc_shift(const float* __restrict__ vol, float* __restrict__ padded, int box) {
  const size_t total = (size_t)box * box * box;
  const int m = 2 * box, half = box / 2;
  const size_t mm = (size_t)m * m;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % box), y = (int)((t / box) % box), z = (int)(t / ((size_t)box * box));
    const float fz = fftfreq_shifted_f32(z + half, m), fy = fftfreq_shifted_f32(y + half, m),
                fx = fftfreq_shifted_f32(x + half, m);
    const float w = sinc2_f32(__fmul_rn(fz, fz), __fmul_rn(fy, fy), __fmul_rn(fx, fx));
    const int zs = (z + 3 * half) % m, ys = (y + 3 * half) % m, xs = (x + 3 * half) % m;
    padded[(size_t)zs * mm + (size_t)ys * m + xs] = __fmul_rn(vol[t], w);
  }
}
}  // namespace

cudaError_t launch_pad_sinc_shift(cudaStream_t st, const float* vol, float* padded, int box) {
  const size_t total = (size_t)box * box * box;
  int grid = (int)((total + 255) / 256);
  if (grid > 152 * 32) grid = 152 * 32;
  pad_sinc_shift<<<grid, 256, 0, st>>>(vol, padded, box);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// gisapr_deposit_noalloc: the deposit entry point for callers that cannot
// allocate device memory.
//
// gisapr_deposit keeps its per-atom records (48 bytes per atom) in a buffer
// the context grows with cudaMalloc. Some callers cannot do that: a host
// whose device memory is handed out by another framework's pool and must not
// change size, code running while a CUDA graph is being captured, or a
// latency-bound loop that cannot afford the device synchronisation a
// cudaMalloc implies. This variant keeps the records in a fixed array in the
// library's own device memory instead, so it allocates nothing and needs no
// context. Every GPU that loads the library holds that array (3 MiB) until
// the process exits.
// ---------------------------------------------------------------------------
#include <mutex>
#include <string>

#include "../../include/gisapr_gb300.h"

void gisapr_internal_set_error(const char* msg);

namespace {

// Largest atom count one call accepts.
constexpr int kNoAllocMaxAtoms = 65536;
static __device__ __align__(256) AtomRec g_noalloc_atoms[kNoAllocMaxAtoms];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

int noalloc_fail(int code, const std::string& msg) {
  gisapr_internal_set_error(msg.c_str());
  return code;
}

}  // namespace

extern "C" int gisapr_deposit_noalloc(void* stream, const float* xyz, const float* numbers, int n_atoms,
                                      float* volume, int box, int width, double apix, double rp, double kn) {
  if (!volume) return noalloc_fail(GISAPR_ERR_ARGUMENT, "volume is NULL");
  if (n_atoms < 0 || (n_atoms > 0 && (!xyz || !numbers)))
    return noalloc_fail(GISAPR_ERR_ARGUMENT, "atom arrays are NULL or n_atoms < 0");
  if (n_atoms > kNoAllocMaxAtoms)
    return noalloc_fail(GISAPR_ERR_ARGUMENT,
                        "gisapr_deposit_noalloc accepts at most " + std::to_string(kNoAllocMaxAtoms) +
                            " atoms per call, got " + std::to_string(n_atoms) +
                            " (split the atoms over several calls or use gisapr_deposit)");
  if (box < 1 || box > 1024) return noalloc_fail(GISAPR_ERR_ARGUMENT, "box out of range");
  if (width < 3) return noalloc_fail(GISAPR_ERR_ARGUMENT, "width must be >= 3 (insufficient sampling)");
  if (!(apix > 0.0) || !(rp > 0.0) || !(kn > 0.0) || !isfinite(apix) || !isfinite(rp) || !isfinite(kn))
    return noalloc_fail(GISAPR_ERR_ARGUMENT, "apix, rp and kn must be positive and finite");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(GISAPR_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return noalloc_fail(GISAPR_ERR_UNSUPPORTED, "device index too large");
  void* recs = nullptr;
  {
    // First call on a device: resolve the device address of the record array
    // with that device current. Host code must not use the symbol itself.
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_atoms);
      if (e != cudaSuccess || !p)
        return noalloc_fail(GISAPR_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      // Under lazy module loading a kernel is loaded on its first launch,
      // which could fall inside a later stream capture; querying both
      // kernels' attributes here loads them now, even for an empty call.
      cudaFuncAttributes fa;
      e = cudaFuncGetAttributes(&fa, atoms_prepare);
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, splat_bricks);
      if (e != cudaSuccess)
        return noalloc_fail(GISAPR_ERR_CUDA, std::string("cudaFuncGetAttributes: ") + cudaGetErrorString(e));
      g_noalloc_ptr[dev] = p;
    }
    recs = g_noalloc_ptr[dev];
  }
  if (n_atoms == 0) return GISAPR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  // Every record a call reads is written first by atoms_prepare in the same
  // call, so nothing left from an earlier call needs clearing.
  e = launch_atoms_prepare(st, xyz, numbers, n_atoms, 0, nullptr, nullptr, nullptr, box, width, apix, kn, recs);
  if (e != cudaSuccess) return noalloc_fail(GISAPR_ERR_CUDA, std::string("atoms_prepare: ") + cudaGetErrorString(e));
  e = launch_splat_bricks(st, recs, n_atoms, volume, volume, nullptr, box, rp);
  if (e != cudaSuccess) return noalloc_fail(GISAPR_ERR_CUDA, std::string("splat_bricks: ") + cudaGetErrorString(e));
  return GISAPR_OK;
}

// ---------------------------------------------------------------------------
// Binned splat (the context entry points): 8^3 bricks, one thread per voxel.
//
// atoms_prepare_binned computes each atom's record as atoms_prepare does and
// appends the atom's index to every 8^3 brick its clipped cube touches
// (fixed capacity per brick; a brick whose list overflows walks every atom in
// input order instead). The
// splat CTA of a brick sorts its list by atom index, so every voxel still
// sums its atoms in input order, and each thread adds the atoms covering its
// voxel. Work is spread over box^3 threads instead of one thread per 16-voxel
// column, which matters because atoms crowd the centre of the box.
// ---------------------------------------------------------------------------
namespace {

constexpr int kBin = 8;

__global__ void atoms_prepare_binned(const float* __restrict__ xyz, const float* __restrict__ numbers, int n,
                                     int transform, const float* __restrict__ pivot,
                                     const double* __restrict__ rot, const double* __restrict__ shift, int box,
                                     int width, double apix, double kn, AtomRec* __restrict__ out,
                                     int* __restrict__ counts, int* __restrict__ lists, int cap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // same record as atoms_prepare
  float c[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  float q[3];
  if (transform) {
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = (double)__fsub_rn(c[k], pivot[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double mm = d[0] * rot[0 * 3 + k];
      mm = fma(d[1], rot[1 * 3 + k], mm);
      mm = fma(d[2], rot[2 * 3 + k], mm);
      q[k] = (float)pdb_8_3(mm + (double)pivot[k] + shift[k]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = c[k];
  }
  float p[3];
  int lo[3], hi[3];
  bool inside = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[k] = (float)((double)q[k] / apix + (double)(box / 2));
    lo[k] = round_away_f64((double)__fsub_rn(p[k], (float)width));
    hi[k] = round_away_f64((double)__fadd_rn(p[k], (float)width));
    inside = inside && (lo[k] < box) && (hi[k] >= 0);
    lo[k] = max(lo[k], 0);
    hi[k] = min(hi[k], box - 1);
  }
  const float z = numbers[i];
  const double zk = (double)z * kn;
  float zk_hi = (float)zk, zk_lo = (float)(zk - (double)zk_hi);
  const bool live = inside && z != 0.0f && isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]) &&
                    hi[0] > lo[0] && hi[1] > lo[1] && hi[2] > lo[2];
  if (!live) { zk_hi = 0.0f; zk_lo = 0.0f; }
  AtomRec r;
  r.px = p[0]; r.py = p[1]; r.pz = p[2];
  r.lx = lo[0]; r.ly = lo[1]; r.lz = lo[2];
  r.ux = hi[0]; r.uy = hi[1]; r.uz = hi[2];
  r.zk_hi = zk_hi; r.zk_lo = zk_lo; r.pad = 0;
  out[i] = r;
  if (!live) return;
  const int nb = (box + kBin - 1) / kBin;
  for (int bz = lo[2] / kBin; bz <= (hi[2] - 1) / kBin; ++bz)
    for (int by = lo[1] / kBin; by <= (hi[1] - 1) / kBin; ++by)
      for (int bx = lo[0] / kBin; bx <= (hi[0] - 1) / kBin; ++bx) {
        const int b = (bz * nb + by) * nb + bx;
        const int slot = atomicAdd(counts + b, 1);
        if (slot < cap) lists[(size_t)b * cap + slot] = i;
      }
}

__global__ void __launch_bounds__(512)
splat_binned(const AtomRec* __restrict__ atoms, int n_atoms, const int* __restrict__ counts,
             const int* __restrict__ lists, int cap, const float* initial, float* out,
             float* __restrict__ padded, int box, float rp_hi, float rp_lo) {
  extern __shared__ int s_ids[];  // cap entries (power of two >= count for the sort)
  __shared__ AtomRec s_rec[64];
  const int nb = (box + kBin - 1) / kBin;
  const int b = blockIdx.x;
  const int bz = b / (nb * nb), by = (b / nb) % nb, bx = b % nb;
  const int x = bx * kBin + (threadIdx.x & 7), y = by * kBin + ((threadIdx.x >> 3) & 7),
            z = bz * kBin + (threadIdx.x >> 6);
  const bool ok = x < box && y < box && z < box;
  const size_t vi = ((size_t)z * box + y) * box + x;
  float acc = (ok && initial != nullptr) ? initial[vi] : 0.0f;
  // A brick whose list overflowed walks every atom in input order instead.
  const bool full_scan = counts[b] > cap;
  const int cnt = full_scan ? n_atoms : counts[b];
  // sort size: the next power of two >= cnt (cnt <= cap here); 0 in full-scan mode
  int pw = 0;
  if (!full_scan) {
    pw = 1;
    while (pw < cnt) pw <<= 1;
  }
  for (int t = threadIdx.x; t < pw; t += blockDim.x) s_ids[t] = t < cnt ? lists[(size_t)b * cap + t] : INT_MAX;
  __syncthreads();
  // bitonic sort: the atomics appended in arbitrary order
  for (int k = 2; !full_scan && k <= pw; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < pw; t += blockDim.x) {
        const int o = t ^ j;
        if (o > t) {
          const int a = s_ids[t], c = s_ids[o];
          const bool up = (t & k) == 0;
          if ((a > c) == up) { s_ids[t] = c; s_ids[o] = a; }
        }
      }
      __syncthreads();
    }
  const float fx = (float)x, fy = (float)y, fz = (float)z;
  for (int base = 0; base < cnt; base += 64) {
    const int nchunk = min(64, cnt - base);
    __syncthreads();
    if (threadIdx.x < nchunk) s_rec[threadIdx.x] = atoms[full_scan ? base + threadIdx.x : s_ids[base + threadIdx.x]];
    __syncthreads();
    for (int t = 0; t < nchunk; ++t) {
      const AtomRec a = s_rec[t];
      if ((a.zk_hi == 0.0f && a.zk_lo == 0.0f) || x < a.lx || x >= a.ux || y < a.ly || y >= a.uy || z < a.lz ||
          z >= a.uz)
        continue;
      const float dx = __fsub_rn(fx, a.px), dy = __fsub_rn(fy, a.py), dz = __fsub_rn(fz, a.pz);
      const float rr = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
      const float ph = __fmul_rn(rr, rp_hi);
      const float pe = __fmaf_rn(rr, rp_hi, -ph);
      const float expo = -__fadd_rn(ph, __fmaf_rn(rr, rp_lo, pe));
      const float e = expf(expo);
      const float vh = __fmul_rn(a.zk_hi, e);
      const float ve = __fmaf_rn(a.zk_hi, e, -vh);
      acc = __fadd_rn(acc, __fadd_rn(vh, __fmaf_rn(a.zk_lo, e, ve)));
    }
  }
  if (!ok) return;
  if (out != nullptr) out[vi] = acc;
  if (padded != nullptr) {
    const int m = 2 * box, half = box / 2;
    const float fzv = fftfreq_shifted_f32(z + half, m), fyv = fftfreq_shifted_f32(y + half, m),
                fxv = fftfreq_shifted_f32(x + half, m);
    const float w = sinc2_f32(__fmul_rn(fzv, fzv), __fmul_rn(fyv, fyv), __fmul_rn(fxv, fxv));
    const int zs = (z + 3 * half) % m, ys = (y + 3 * half) % m, xs = (x + 3 * half) % m;
    padded[((size_t)zs * m + ys) * m + xs] = __fmul_rn(acc, w);
  }
}

}  // namespace

int splat_bin_cap() { return 1024; }
int splat_bin_count(int box) {
  const int nb = (box + kBin - 1) / kBin;
  return nb * nb * nb;
}

cudaError_t launch_splat_binned(cudaStream_t st, const float* xyz, const float* numbers, int n, int transform,
                                const float* pivot, const double* rot, const double* shift, const float* initial,
                                float* out, float* padded, int box, int width, double apix, double rp, double kn,
                                void* atom_recs, int* counts, int* lists) {
  const int nbricks = splat_bin_count(box), cap = splat_bin_cap();
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * nbricks, st);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    // 64 threads a block: a few thousand atoms spread over many SMs (the
    // FP64 pose and 8.3 rounding are long dependent chains per atom)
    atoms_prepare_binned<<<(n + 63) / 64, 64, 0, st>>>(xyz, numbers, n, transform, pivot, rot, shift, box,
                                                           width, apix, kn, (AtomRec*)atom_recs, counts, lists,
                                                           cap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const float rp_hi = (float)rp, rp_lo = (float)(rp - (double)rp_hi);
  splat_binned<<<nbricks, 512, cap * sizeof(int), st>>>((const AtomRec*)atom_recs, n, counts, lists, cap,
                                                       initial, out, padded, box, rp_hi, rp_lo);
  return cudaGetLastError();
}
