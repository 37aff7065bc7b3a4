// Geometric restraint of a moved chain against the fixed main body
// (func_check_boundary_for_testing_v8.py:62-126).
//
// Once per job the main body's density is thresholded into a voxel mask and
// its exact squared Euclidean distance transform is built: d2(v) = the
// squared distance from voxel v to the nearest mask voxel (0 on the mask),
// the integer whose square root scipy's distance_transform_edt(~mask)
// returns. The transform is separable: three passes, one per axis, each
//   g(p) = min over q of (p - q)^2 + f(q)
// along every line of the axis (f = 0 on mask voxels and "infinite"
// elsewhere for the first pass, the previous pass's output after that).
// Each pass stages a tile of 32 lines in shared memory and evaluates the
// minimum directly over the line; integer arithmetic makes the result exact.
//
// Per candidate the moved chain is splatted onto an all-zero scratch volume
// (the ordinary deposit kernel), then restraint_reduce walks the chain's
// bounding box once: voxels above the threshold count as overlap where the
// mask is set and contribute their d2 to a minimum; every voxel it reads is
// zeroed again, so the scratch volume is all-zero for the next candidate.
#include "common.cuh"

#include <climits>

namespace {

constexpr int kEdtInf = 1 << 29;  // above any squared distance of a 1024^3 grid (3 * 1023^2)
constexpr int kTileLines = 32;
constexpr int kEdtThreads = 256;

// Pass along x (the contiguous axis). Block: 32 consecutive lines (y0..y0+31
// of one z), the whole x extent. The first pass reads the density and
// writes the mask too.
__global__ void __launch_bounds__(kEdtThreads) edt_pass_x(const float* __restrict__ density, float threshold,
                                                           unsigned char* __restrict__ mask,
                                                           int* __restrict__ out, int box) {
  extern __shared__ int s_f[];  // [kTileLines][box]
  const int z = blockIdx.y, y0 = blockIdx.x * kTileLines;
  const int lines = min(kTileLines, box - y0);
  for (int i = threadIdx.x; i < lines * box; i += blockDim.x) {
    const int l = i / box, x = i - l * box;
    const size_t v = ((size_t)z * box + (y0 + l)) * box + x;
    const bool on = density[v] > threshold;
    mask[v] = on ? 1 : 0;
    s_f[l * box + x] = on ? 0 : kEdtInf;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < lines * box; i += blockDim.x) {
    const int l = i / box, p = i - l * box;
    const int* f = s_f + l * box;
    int best = kEdtInf;
    for (int q = 0; q < box; ++q) {
      const int d = p - q;
      best = min(best, f[q] + d * d);
    }
    out[((size_t)z * box + (y0 + l)) * box + p] = best >= kEdtInf ? kEdtInf : best;
  }
}

// Pass along y (axis 1) or z (axis 2). Block: 32 consecutive x of one line
// index of the other axis, the whole extent of the pass axis; loads and
// stores are coalesced along x.
__global__ void __launch_bounds__(kEdtThreads) edt_pass_yz(const int* __restrict__ in, int* __restrict__ out,
                                                            int box, int axis) {
  extern __shared__ int s_f[];  // [box][kTileLines]
  const int x0 = blockIdx.x * kTileLines, other = blockIdx.y;
  const int lanes = min(kTileLines, box - x0);
  // element (p, x) of the tile: voxel (z, y, x) with p on the pass axis
  const size_t stride_p = axis == 1 ? (size_t)box : (size_t)box * box;
  const size_t base = axis == 1 ? (size_t)other * box * box : (size_t)other * box;
  for (int i = threadIdx.x; i < box * kTileLines; i += blockDim.x) {
    const int p = i / kTileLines, l = i - p * kTileLines;
    if (l < lanes) s_f[p * kTileLines + l] = in[base + p * stride_p + x0 + l];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < box * kTileLines; i += blockDim.x) {
    const int p = i / kTileLines, l = i - p * kTileLines;
    if (l >= lanes) continue;
    int best = kEdtInf;
    for (int q = 0; q < box; ++q) {
      const int d = p - q;
      best = min(best, s_f[q * kTileLines + l] + d * d);
    }
    out[base + p * stride_p + x0 + l] = best >= kEdtInf ? kEdtInf : best;
  }
}

struct Box3 {
  int lo[3], hi[3];  // z, y, x; half-open
};

// out[0] += overlap voxels, out[1] = min d2 over chain voxels, out[2] |= any
// chain voxel. Zeroes every voxel of the box it reads.
__global__ void __launch_bounds__(256) restraint_reduce(float* __restrict__ volume,
                                                         const unsigned char* __restrict__ mask,
                                                         const int* __restrict__ d2, int box, Box3 b,
                                                         float threshold, int* __restrict__ out) {
  const int ex = b.hi[2] - b.lo[2], ey = b.hi[1] - b.lo[1], ez = b.hi[0] - b.lo[0];
  const long long total = (long long)ex * ey * ez;
  int count = 0, dmin = INT_MAX, any = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % ex), y = (int)((t / ex) % ey), z = (int)(t / ((long long)ex * ey));
    const size_t v = ((size_t)(b.lo[0] + z) * box + (b.lo[1] + y)) * box + (b.lo[2] + x);
    const float val = volume[v];
    if (val > threshold) {
      any = 1;
      count += mask[v];
      dmin = min(dmin, d2[v]);
    }
    if (val != 0.0f) volume[v] = 0.0f;
  }
  // warp then block reduction, one atomic of each kind per block
  for (int o = 16; o > 0; o >>= 1) {
    count += __shfl_xor_sync(0xffffffffu, count, o);
    dmin = min(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    any |= __shfl_xor_sync(0xffffffffu, any, o);
  }
  __shared__ int s_c[8], s_d[8], s_a[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { s_c[warp] = count; s_d[warp] = dmin; s_a[warp] = any; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0, d = INT_MAX, a = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { c += s_c[w]; d = min(d, s_d[w]); a |= s_a[w]; }
    if (c) atomicAdd(out + 0, c);
    if (d != INT_MAX) atomicMin(out + 1, d);
    if (a) atomicOr(out + 2, a);
  }
}

__global__ void restraint_init(int* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[3 * i + 0] = 0;
    out[3 * i + 1] = INT_MAX;
    out[3 * i + 2] = 0;
  }
}

}  // namespace

size_t edt_smem_bytes(int box) { return (size_t)kTileLines * box * sizeof(int); }

cudaError_t launch_restraint_edt(cudaStream_t st, const float* density, float threshold, unsigned char* mask,
                                 int* d2, int* scratch, int box) {
  const size_t smem = edt_smem_bytes(box);
  cudaError_t e = cudaFuncSetAttribute(edt_pass_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(edt_pass_yz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tiles = (box + kTileLines - 1) / kTileLines;
  edt_pass_x<<<dim3(tiles, box), kEdtThreads, smem, st>>>(density, threshold, mask, d2, box);
  edt_pass_yz<<<dim3(tiles, box), kEdtThreads, smem, st>>>(d2, scratch, box, 1);
  edt_pass_yz<<<dim3(tiles, box), kEdtThreads, smem, st>>>(scratch, d2, box, 2);
  return cudaGetLastError();
}

cudaError_t launch_restraint_init(cudaStream_t st, int* out, int n) {
  restraint_init<<<(n + 127) / 128, 128, 0, st>>>(out, n);
  return cudaGetLastError();
}

cudaError_t launch_restraint_reduce(cudaStream_t st, float* volume, const unsigned char* mask, const int* d2,
                                    int box, const int* lo, const int* hi, float threshold, int* out,
                                    int sm_count) {
  Box3 b;
  long long total = 1;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = lo[a];
    b.hi[a] = hi[a];
    total *= (long long)(hi[a] - lo[a]);
  }
  if (total <= 0) return cudaSuccess;
  long long blocks = (total + 255) / 256;
  const long long cap = 4LL * sm_count;
  if (blocks > cap) blocks = cap;
  restraint_reduce<<<(int)blocks, 256, 0, st>>>(volume, mask, d2, box, b, threshold, out);
  return cudaGetLastError();
}
