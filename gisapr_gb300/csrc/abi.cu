// C ABI entry points (include/gisapr_gb300.h): argument checks, per-device
// context (twiddle and radial-bin tables, cuFFT plans, scratch) and launches.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gisapr_gb300.h"
#include "common.cuh"

// ---- launchers defined in the other translation units
cudaError_t launch_atoms_prepare(cudaStream_t, const float*, const float*, int, int, const float*,
                                 const double*, const double*, int, int, double, double, void*);
size_t atom_record_bytes();
cudaError_t launch_splat_bricks(cudaStream_t, const void*, int, const float*, float*, float*, int,
                                double);
cudaError_t launch_pad_sinc_shift(cudaStream_t, const float*, float*, int);
int splat_bin_cap();
int splat_bin_count(int box);
cudaError_t launch_splat_binned(cudaStream_t, const float*, const float*, int, int, const float*, const double*,
                                const double*, const float*, float*, float*, int, int, double, double, double, void*,
                                int*, int*);
size_t project_scratch_elems(int N, int nb);
size_t project_smem_bytes(int N, int n_bins);
cudaError_t launch_project_templates(cudaStream_t, const float2*, const float*, const int*, int,
                                     const int*, const float*, const float*, const int*, const int*,
                                     const float*, int, const float2*, const float2*, float2*, float2*, int,
                                     int, int);
size_t project_smem_bytes_fast(int N, int n_bins, int nb);
cudaError_t launch_project_templates_fast(cudaStream_t, const float2*, const float*, const int*, int,
                                          const int*, const float*, const float*, const int*, const int*,
                                          const float*, int, const float2*, float2*, int, int, int, float2*,
                                          float2*, int*, unsigned);
size_t project_blocked_elems(int N);
size_t project_slice_elems(int N, int n_build);
cudaError_t launch_project_templates_planes(cudaStream_t, const float2*, const float*, const int*, int,
                                            const int*, const float*, const float*, const int*, const int*,
                                            const float*, int, const float2*, const float2*, float2*, float2*,
                                            int, int, int, float2*, float2*, int);
size_t project_flat_plane_elems(int N, int n);
size_t vfft_scratch_elems(int N);
cudaError_t launch_volume_spectrum_blocked(cudaStream_t, const float*, int, float2*, float2*, const float2*);
cudaError_t launch_packed_ctf(cudaStream_t, const float*, const float*, const float*, int,
                              const float*, const float*, const float*, const float*, int, float,
                              float, float, float, float, float*);
size_t prepare_scratch_elems(int N, int nb);
cudaError_t launch_prepare_particles(cudaStream_t, const float*, int, int, const int*, const void*,
                                     const float*, const float*, float2*, float2*, int,
                                     const float2*, const float2*, int, int);
int correlate_cluster_size(int n);
size_t correlate_smem_bytes(int n, int n_psi, int crop, int cluster);
cudaError_t launch_correlate_plain(cudaStream_t, const float2*, const float2*, const int*,
                                   const int*, int, int, int, int, const float2*, const float2*,
                                   float*, int*, int*, int, long long, int, int, const unsigned char*);
cudaError_t launch_particle_results(cudaStream_t, const int*, const float*, const int*, const int*,
                                    int, int, int*, int*, float*, int*, int*, float*, int, const unsigned char*);
cudaError_t launch_score_sum(cudaStream_t, const int*, const float*, int, double*, int, const unsigned char*);
size_t edt_smem_bytes(int box);
cudaError_t launch_restraint_edt(cudaStream_t, const float*, float, unsigned char*, int*, int*, int);
cudaError_t launch_restraint_init(cudaStream_t, int*, int);
cudaError_t launch_restraint_reduce(cudaStream_t, float*, const unsigned char*, const int*, int, const int*,
                                    const int*, float, int*, int);
cudaError_t launch_ingest_load(cudaStream_t, const float*, int, int, int, const int*, int, int, double2*, int);
cudaError_t launch_ingest_spectrum_divide(cudaStream_t, double2*, int, int, const int*, const int*, const double*,
                                          int);
cudaError_t launch_ingest_normalize(cudaStream_t, double2*, int, int, int, double);
cudaError_t launch_ingest_scale_mask(cudaStream_t, double2*, int, int, const double*, double, int, int);
cudaError_t launch_ingest_store(cudaStream_t, const double2*, int, int, double, float*, int);
int correlate_tc_max_psi();
int correlate_tc_max_n();
size_t correlate_tc_smem_bytes(int n, int crop, int split, int sa, int sb);
bool correlate_tc_rings(int n, int crop, int split, int want_sa, int want_sb, int* sa, int* sb);
long long correlate_tc_bank_halves(int n_slot, int n);
int correlate_tc_plan(const int*, const int*, int, int, int, int, int*, int);
cudaError_t launch_bank_to_operands(cudaStream_t, const float2*, long long, int, int, int, int, int, const float*,
                                    void*, int*);
int correlate_tc_max_cand();
cudaError_t launch_correlate_tc(cudaStream_t, const void*, int, const float2*, const int*, const int*, const int*,
                                int, int, int, int, int, int, int, const float*, const float*, unsigned,
                                const float2*, const float2*, float*, int*, int*, int*, int, int, int);

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(GISAPR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorName(e) + " (" +
                                   cudaGetErrorString(e) + ")");
}

#define GISAPR_CHECK_CUDA(expr, where)          \
  do {                                          \
    cudaError_t _e = (expr);                    \
    if (_e != cudaSuccess) return cuda_fail(_e, where); \
  } while (0)

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct BinTable {
  int* list = nullptr;
  int* ptr = nullptr;
  float* count = nullptr;
  int n_bins = 0;
};

struct CorrTables {
  float2* outer = nullptr;  // [M][C]
  float2* col = nullptr;    // [H][C]
  float2* row = nullptr;    // [n] exp(+2 pi i t / n)
};

}  // namespace

// Lets the other translation units of the library report errors through
// gisapr_last_error().
void gisapr_internal_set_error(const char* msg) { g_last_error = msg; }

struct gisapr_context {
  int device = 0;
  float2* tw = nullptr;   // exp(-2 pi i t / kMaxFftLen), t < kMaxFftLen/2
  float2* tw3 = nullptr;  // exp(-2 pi i t / kMaxFftLen3), t < kMaxFftLen3 (lengths 3 * 2^k)
  std::map<int, std::pair<cufftHandle, float*>> fft;  // box -> (R2C plan, padded input)
  std::map<int, BinTable> bins;                        // N -> radial bins
  std::map<std::pair<int, int>, CorrTables> corr;      // (n, crop) -> twiddles
  DeviceBuffer atoms, bin_counts, bin_lists, proj_scratch, prep_scratch, proj_slices, proj_blocked, vfft_scratch;
  DeviceBuffer proj_status;        // int: set to 1 by a projector plane wait that ran out
  unsigned proj_wait = 1u << 24;   // bound of that wait (attempts)
  int blocked_box = 0;  // box of the blocked spectrum gisapr_volume_spectrum_blocked last wrote (0: none)
  // Buffers replaced by larger ones. They are freed only with the context:
  // a CUDA graph captured before a buffer grew still names the old one, and
  // that buffer stays valid (and large enough for the graph's own sizes).
  // A buffer that grows at least doubles (see ensure), so the retired
  // buffers of one kind hold less memory than the live one.
  std::vector<void*> retired;
  int sm_count = 152;
  std::map<int, int> tune_corr_cluster;  // n -> CTAs per particle in the plain correlation
  std::map<int, int> tune_tc_a, tune_tc_b;  // n -> A / B ring depth of the tensor-core correlation
};

namespace {

int set_device(gisapr_ctx ctx) {
  GISAPR_CHECK_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  return GISAPR_OK;
}

// Make ``b`` hold at least ``bytes``. The first allocation is exact; a
// buffer that has to grow is replaced by one of at least twice its size, so
// a context that sees growing requests keeps less than twice the live
// buffer in total (live plus retired) and the live buffer stays below twice
// the largest request.
int ensure(gisapr_ctx ctx, DeviceBuffer& b, size_t bytes, const char* what) {
  if (b.bytes >= bytes) return GISAPR_OK;
  if (b.ptr) {
    ctx->retired.push_back(b.ptr);
    bytes = std::max(bytes, 2 * b.bytes);
  }
  b.ptr = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e != cudaSuccess) return cuda_fail(e, what);
  b.bytes = bytes;
  return GISAPR_OK;
}

int get_fft(gisapr_ctx ctx, int box, cufftHandle* plan, float** padded) {
  auto it = ctx->fft.find(box);
  if (it != ctx->fft.end()) {
    *plan = it->second.first;
    *padded = it->second.second;
    return GISAPR_OK;
  }
  const int m = 2 * box;
  float* buf = nullptr;
  const size_t bytes = (size_t)m * m * m * sizeof(float);
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(FFT input)");
  // The zero padding outside the centred box is written once and never
  // touched again: the splat and pad kernels only write the box region and
  // an out-of-place R2C leaves its input unchanged.
  e = cudaMemset(buf, 0, bytes);
  if (e != cudaSuccess) { cudaFree(buf); return cuda_fail(e, "cudaMemset(FFT input)"); }
  cufftHandle h;
  cufftResult r = cufftPlan3d(&h, m, m, m, CUFFT_R2C);
  if (r != CUFFT_SUCCESS) {
    cudaFree(buf);
    return fail(GISAPR_ERR_CUFFT, "cufftPlan3d failed with code " + std::to_string((int)r));
  }
  ctx->fft[box] = {h, buf};
  *plan = h;
  *padded = buf;
  return GISAPR_OK;
}

int get_bins(gisapr_ctx ctx, int N, BinTable* out) {
  auto it = ctx->bins.find(N);
  if (it != ctx->bins.end()) { *out = it->second; return GISAPR_OK; }
  const int HC = N / 2 + 1;
  std::vector<int> bin_of(N * HC);
  int max_bin = 0;
  for (int r = 0; r < N; ++r)
    for (int kx = 0; kx < HC; ++kx) {
      const int ky = r < N / 2 ? r : r - N;
      const int b = (int)std::nearbyint(std::sqrt((float)(ky * ky + kx * kx)));
      bin_of[r * HC + kx] = b;
      if (b > max_bin) max_bin = b;
    }
  const int nb = max_bin + 1;
  // full-grid counts, radius of the fftshifted N x N grid (v606:901-913)
  std::vector<float> cnt(nb, 0.f);
  for (int y = 0; y < N; ++y)
    for (int x = 0; x < N; ++x) {
      const int dy = y - N / 2, dx = x - N / 2;
      const int b = (int)std::nearbyint(std::sqrt((float)(dy * dy + dx * dx)));
      if (b < nb) cnt[b] += 1.f;
    }
  std::vector<int> ptr(nb + 1, 0), list(N * HC);
  for (int i = 0; i < N * HC; ++i) ptr[bin_of[i] + 1]++;
  for (int b = 0; b < nb; ++b) ptr[b + 1] += ptr[b];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int i = 0; i < N * HC; ++i) list[fill[bin_of[i]]++] = i;
  BinTable t;
  t.n_bins = nb;
  GISAPR_CHECK_CUDA(cudaMalloc(&t.list, list.size() * sizeof(int)), "cudaMalloc(bins)");
  GISAPR_CHECK_CUDA(cudaMalloc(&t.ptr, ptr.size() * sizeof(int)), "cudaMalloc(bins)");
  GISAPR_CHECK_CUDA(cudaMalloc(&t.count, cnt.size() * sizeof(float)), "cudaMalloc(bins)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice),
                    "cudaMemcpy(bins)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice),
                    "cudaMemcpy(bins)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.count, cnt.data(), cnt.size() * sizeof(float), cudaMemcpyHostToDevice),
                    "cudaMemcpy(bins)");
  ctx->bins[N] = t;
  *out = t;
  return GISAPR_OK;
}

int get_corr_tables(gisapr_ctx ctx, int n, int crop, CorrTables* out) {
  auto key = std::make_pair(n, crop);
  auto it = ctx->corr.find(key);
  if (it != ctx->corr.end()) { *out = it->second; return GISAPR_OK; }
  const int M = n / 16, H = n / 2 + 1, h = crop / 2;
  const double two_pi = 6.283185307179586476925286766559;
  std::vector<float2> outer((size_t)M * crop), col((size_t)H * crop);
  for (int q = 0; q < M; ++q)
    for (int yi = 0; yi < crop; ++yi) {
      const double a = two_pi * (double)q * (double)(yi - h) / (double)n;
      outer[(size_t)q * crop + yi] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  for (int c = 0; c < H; ++c) {
    const double w = (c == 0 || c == n / 2) ? 1.0 : 2.0;
    for (int xi = 0; xi < crop; ++xi) {
      const double a = two_pi * (double)c * (double)(xi - h) / (double)n;
      col[(size_t)c * crop + xi] = make_float2((float)(w * std::cos(a)), (float)(w * std::sin(a)));
    }
  }
  std::vector<float2> row(n);
  for (int t = 0; t < n; ++t) {
    const double a = two_pi * (double)t / (double)n;
    row[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  CorrTables t;
  GISAPR_CHECK_CUDA(cudaMalloc(&t.row, row.size() * sizeof(float2)), "cudaMalloc(corr)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.row, row.data(), row.size() * sizeof(float2), cudaMemcpyHostToDevice),
                    "cudaMemcpy(corr)");
  GISAPR_CHECK_CUDA(cudaMalloc(&t.outer, outer.size() * sizeof(float2)), "cudaMalloc(corr)");
  GISAPR_CHECK_CUDA(cudaMalloc(&t.col, col.size() * sizeof(float2)), "cudaMalloc(corr)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.outer, outer.data(), outer.size() * sizeof(float2), cudaMemcpyHostToDevice),
                    "cudaMemcpy(corr)");
  GISAPR_CHECK_CUDA(cudaMemcpy(t.col, col.data(), col.size() * sizeof(float2), cudaMemcpyHostToDevice),
                    "cudaMemcpy(corr)");
  ctx->corr[key] = t;
  *out = t;
  return GISAPR_OK;
}

int tuned_cluster(gisapr_ctx ctx, int n) {
  auto it = ctx->tune_corr_cluster.find(n);
  return it == ctx->tune_corr_cluster.end() ? 0 : it->second;
}

// Boxes are powers of two from 32 to 256, or 96 and 192 (3 * 2^k: the
// shared-memory transforms run a radix-3 pass over radix-2 sub-transforms).
int check_box(int box) {
  if (!((is_pow2(box) && box >= 32 && box <= 256) || box == 96 || box == 192))
    return fail(GISAPR_ERR_UNSUPPORTED, "box must be a power of two in [32, 256], 96 or 192, got " +
                                            std::to_string(box));
  return GISAPR_OK;
}

int check_newbox(int box, int nb) {
  if (nb <= 0 || nb % 16 != 0 || nb > box)
    return fail(GISAPR_ERR_ARGUMENT, "newbox must be a positive multiple of 16 not above box, got " +
                                         std::to_string(nb));
  return GISAPR_OK;
}

int grid_for(gisapr_ctx ctx, int work, int per_sm) {
  int g = ctx->sm_count * per_sm;
  return work < g ? work : g;
}

}  // namespace

extern "C" {

int gisapr_abi_version(void) { return 100; }

const char* gisapr_last_error(void) { return g_last_error.c_str(); }

int gisapr_context_create(int device, gisapr_ctx* out) {
  if (!out) return fail(GISAPR_ERR_ARGUMENT, "out is NULL");
  *out = nullptr;
  int n_dev = 0;
  GISAPR_CHECK_CUDA(cudaGetDeviceCount(&n_dev), "cudaGetDeviceCount");
  if (device < 0 || device >= n_dev)
    return fail(GISAPR_ERR_ARGUMENT, "device index out of range: " + std::to_string(device));
  GISAPR_CHECK_CUDA(cudaSetDevice(device), "cudaSetDevice");
  gisapr_context* ctx = new gisapr_context();
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  std::vector<float2> tw(kMaxFftLen / 2);
  const double two_pi = 6.283185307179586476925286766559;
  for (int t = 0; t < kMaxFftLen / 2; ++t) {
    const double a = -two_pi * (double)t / (double)kMaxFftLen;
    tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  std::vector<float2> tw3(kMaxFftLen3);
  for (int t = 0; t < kMaxFftLen3; ++t) {
    const double a = -two_pi * (double)t / (double)kMaxFftLen3;
    tw3[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  cudaError_t e = cudaMalloc(&ctx->tw, tw.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(ctx->tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->tw3, tw3.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(ctx->tw3, tw3.data(), tw3.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_fail(e, "context tables");
  }
  *out = ctx;
  return GISAPR_OK;
}

int gisapr_context_destroy(gisapr_ctx ctx) {
  if (!ctx) return GISAPR_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (auto& kv : ctx->fft) { cufftDestroy(kv.second.first); cudaFree(kv.second.second); }
  for (auto& kv : ctx->bins) { cudaFree(kv.second.list); cudaFree(kv.second.ptr); cudaFree(kv.second.count); }
  for (auto& kv : ctx->corr) { cudaFree(kv.second.outer); cudaFree(kv.second.col); }
  cudaFree(ctx->atoms.ptr);
  cudaFree(ctx->bin_counts.ptr);
  cudaFree(ctx->bin_lists.ptr);
  cudaFree(ctx->proj_scratch.ptr);
  cudaFree(ctx->proj_slices.ptr);
  cudaFree(ctx->proj_blocked.ptr);
  cudaFree(ctx->prep_scratch.ptr);
  cudaFree(ctx->vfft_scratch.ptr);
  cudaFree(ctx->proj_status.ptr);
  cudaFree(ctx->tw);
  for (void* p : ctx->retired) cudaFree(p);
  cudaFree(ctx->tw3);
  delete ctx;
  return GISAPR_OK;
}

static int deposit_common(gisapr_ctx ctx, void* stream, const float* xyz, const float* numbers, int n,
                          int transform, const float* pivot, const double* rot, const double* shift,
                          const float* initial, float* out, float* padded, int box, int width,
                          double apix, double rp, double kn) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n < 0 || (n > 0 && (!xyz || !numbers)))
    return fail(GISAPR_ERR_ARGUMENT, "atom arrays are NULL or n_atoms < 0");
  if (box < 1 || box > 1024) return fail(GISAPR_ERR_ARGUMENT, "box out of range");
  if (width < 3) return fail(GISAPR_ERR_ARGUMENT, "width must be >= 3 (insufficient sampling)");
  if (!(apix > 0.0) || !std::isfinite(apix) || !std::isfinite(rp) || !std::isfinite(kn))
    return fail(GISAPR_ERR_ARGUMENT, "apix, rp and kn must be positive and finite");
  if (transform && (!pivot || !rot || !shift)) return fail(GISAPR_ERR_ARGUMENT, "pose arrays are NULL");
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  rc = ensure(ctx, ctx->atoms, (size_t)(n > 0 ? n : 1) * atom_record_bytes(), "cudaMalloc(atoms)");
  if (rc) return rc;
  const size_t nbricks = (size_t)splat_bin_count(box);
  rc = ensure(ctx, ctx->bin_counts, nbricks * sizeof(int), "cudaMalloc(brick counts)");
  if (rc) return rc;
  rc = ensure(ctx, ctx->bin_lists, nbricks * splat_bin_cap() * sizeof(int), "cudaMalloc(brick lists)");
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_splat_binned(st, xyz, numbers, n, transform, pivot, rot, shift, initial, out, padded,
                                        box, width, apix, rp, kn, ctx->atoms.ptr, (int*)ctx->bin_counts.ptr,
                                        (int*)ctx->bin_lists.ptr),
                    "splat");
  return GISAPR_OK;
}

int gisapr_deposit(gisapr_ctx ctx, void* stream, const float* xyz, const float* numbers, int n_atoms,
                   float* volume, int box, int width, double apix, double rp, double kn) {
  if (!volume) return fail(GISAPR_ERR_ARGUMENT, "volume is NULL");
  return deposit_common(ctx, stream, xyz, numbers, n_atoms, 0, nullptr, nullptr, nullptr, volume, volume,
                        nullptr, box, width, apix, rp, kn);
}

int gisapr_deposit_moved(gisapr_ctx ctx, void* stream, const float* xyz, const float* numbers,
                         int n_atoms, const float* pivot, const double* rot, const double* shift,
                         const float* fixed, float* out, int write_padded, int box, int width,
                         double apix, double rp, double kn) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (!out && !write_padded) return fail(GISAPR_ERR_ARGUMENT, "nothing to write: out is NULL and write_padded is 0");
  float* padded = nullptr;
  if (write_padded) {
    int rc = check_box(box);
    if (rc) return rc;
    rc = set_device(ctx);
    if (rc) return rc;
    cufftHandle plan;
    rc = get_fft(ctx, box, &plan, &padded);
    if (rc) return rc;
  }
  return deposit_common(ctx, stream, xyz, numbers, n_atoms, 1, pivot, rot, shift, fixed, out, padded, box,
                        width, apix, rp, kn);
}

int gisapr_volume_spectrum(gisapr_ctx ctx, void* stream, const float* volume, int box, float* spectrum) {
  if (!ctx || !spectrum) return fail(GISAPR_ERR_ARGUMENT, "context or spectrum is NULL");
  int rc = check_box(box);
  if (rc) return rc;
  rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cufftHandle plan;
  float* padded = nullptr;
  rc = get_fft(ctx, box, &plan, &padded);
  if (rc) return rc;
  if (volume) GISAPR_CHECK_CUDA(launch_pad_sinc_shift(st, volume, padded, box), "pad_sinc_shift");
  cufftResult r = cufftSetStream(plan, st);
  if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftSetStream failed");
  r = cufftExecR2C(plan, (cufftReal*)padded, (cufftComplex*)spectrum);
  if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftExecR2C failed with code " + std::to_string((int)r));
  return GISAPR_OK;
}

// box-256 templates per rows_inverse + general-kernel pair (planes of 526 KB)
constexpr int kPlaneChunk = 4096;

int gisapr_project_launches(int box, int n_build) {
  if (!((is_pow2(box) && box >= 32 && box <= 256) || box == 96 || box == 192)) return -1;
  if (n_build <= 0) return 0;
  if (box <= 128 && is_pow2(box)) return 3;  // blocked copy, gather + row inverse, template tail
  if (box == 256) return 1 + 2 * ((n_build + kPlaneChunk - 1) / kPlaneChunk);
  return 1;
}

int gisapr_volume_spectrum_blocked(gisapr_ctx ctx, void* stream, const float* volume, int box) {
  if (!ctx || !volume) return fail(GISAPR_ERR_ARGUMENT, "context or volume is NULL");
  if (!(is_pow2(box) && box >= 32 && box <= 256))
    return fail(GISAPR_ERR_UNSUPPORTED, "the blocked volume transform takes a power-of-two box in [32, 256]");
  int rc = set_device(ctx);
  if (rc) return rc;
  rc = ensure(ctx, ctx->vfft_scratch, vfft_scratch_elems(box) * sizeof(float2), "cudaMalloc(volume transform)");
  if (rc) return rc;
  rc = ensure(ctx, ctx->proj_blocked, project_blocked_elems(box) * sizeof(float2), "cudaMalloc(blocked spectrum)");
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_volume_spectrum_blocked((cudaStream_t)stream, volume, box, (float2*)ctx->vfft_scratch.ptr,
                                                   (float2*)ctx->proj_blocked.ptr, ctx->tw),
                    "volume_spectrum_blocked");
  ctx->blocked_box = box;
  return GISAPR_OK;
}

// The projector's status word, allocated and zeroed on the context's first
// shared-memory projector call (before any stream capture of that call).
static int status_word(gisapr_ctx ctx) {
  if (ctx->proj_status.ptr) return GISAPR_OK;
  const int rc = ensure(ctx, ctx->proj_status, sizeof(int), "cudaMalloc(projector status)");
  if (rc) return rc;
  GISAPR_CHECK_CUDA(cudaMemset(ctx->proj_status.ptr, 0, sizeof(int)), "cudaMemset(projector status)");
  return GISAPR_OK;
}

int gisapr_set_projector_wait(gisapr_ctx ctx, long long attempts) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "ctx is NULL");
  ctx->proj_wait = attempts < 0 ? (1u << 24) : (unsigned)std::min<long long>(attempts, 0xffffffffLL);
  return GISAPR_OK;
}

int gisapr_projector_status(gisapr_ctx ctx, void* stream, int* value) {
  if (!ctx || !value) return fail(GISAPR_ERR_ARGUMENT, "ctx or value is NULL");
  *value = 0;
  if (!ctx->proj_status.ptr) return GISAPR_OK;
  int rc = set_device(ctx);
  if (rc) return rc;
  const cudaStream_t st = (cudaStream_t)stream;
  int h = 0;
  GISAPR_CHECK_CUDA(cudaMemcpyAsync(&h, ctx->proj_status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st),
                    "cudaMemcpyAsync(projector status)");
  GISAPR_CHECK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (h != 0) {
    GISAPR_CHECK_CUDA(cudaMemsetAsync(ctx->proj_status.ptr, 0, sizeof(int), st), "cudaMemsetAsync(projector status)");
    GISAPR_CHECK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  }
  *value = h;
  return GISAPR_OK;
}

int gisapr_project_templates(gisapr_ctx ctx, void* stream, const float* spectrum, int box,
                             const float* rot, const int* dirs, int n_build, const int* out_slot,
                             const float* mask, const float* fsc, int newbox, float* bank) {
  if (!ctx || !rot || !dirs || !fsc || !bank)
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  int rc = check_box(box);
  if (rc) return rc;
  if (!spectrum && ctx->blocked_box != box)
    return fail(GISAPR_ERR_ARGUMENT, "spectrum is NULL and no blocked spectrum of this box was written "
                                     "(gisapr_volume_spectrum_blocked) on this context");
  rc = check_newbox(box, newbox);
  if (rc) return rc;
  if (n_build < 0) return fail(GISAPR_ERR_ARGUMENT, "n_build < 0");
  if (n_build == 0) return GISAPR_OK;
  rc = set_device(ctx);
  if (rc) return rc;
  BinTable bt;
  rc = get_bins(ctx, box, &bt);
  if (rc) return rc;
  if (box <= 128 && is_pow2(box)) {
    // whole template in shared memory, one CTA per SM
    const int grid = grid_for(ctx, n_build, 1);
    if (n_build > 65535) return fail(GISAPR_ERR_ARGUMENT, "at most 65535 templates per call");
    rc = ensure(ctx, ctx->proj_slices, project_slice_elems(box, n_build) * sizeof(float2), "cudaMalloc(planes)");
    if (rc) return rc;
    rc = ensure(ctx, ctx->proj_blocked, project_blocked_elems(box) * sizeof(float2), "cudaMalloc(blocked spectrum)");
    if (rc) return rc;
    rc = status_word(ctx);
    if (rc) return rc;
    GISAPR_CHECK_CUDA(launch_project_templates_fast((cudaStream_t)stream, (const float2*)spectrum, rot, dirs,
                                                    n_build, out_slot, mask, fsc, bt.list, bt.ptr, bt.count,
                                                    bt.n_bins, ctx->tw, (float2*)bank, grid, box, newbox,
                                                    (float2*)ctx->proj_slices.ptr, (float2*)ctx->proj_blocked.ptr,
                                                    (int*)ctx->proj_status.ptr, ctx->proj_wait),
                      "project_templates");
    ctx->blocked_box = box;
    return GISAPR_OK;
  }
  // CTAs per SM of the general path (measured on GB300): smaller boxes fill
  // the SM with more CTAs while their scratch planes still fit L2
  const int grid = grid_for(ctx, n_build, box == 96 ? 6 : (box == 192 ? 3 : 2));
  rc = ensure(ctx, ctx->proj_scratch, (size_t)grid * project_scratch_elems(box, newbox) * sizeof(float2),
              "cudaMalloc(projector scratch)");
  if (rc) return rc;
  if (box == 256) {
    // the gather and pass A in their own high-occupancy kernel, from the
    // blocked spectrum, at most 4,096 planes (2.2 GB) at a time
    const int chunk = std::min(n_build, kPlaneChunk);
    rc = ensure(ctx, ctx->proj_slices, project_flat_plane_elems(box, chunk) * sizeof(float2), "cudaMalloc(planes)");
    if (rc) return rc;
    rc = ensure(ctx, ctx->proj_blocked, project_blocked_elems(box) * sizeof(float2), "cudaMalloc(blocked spectrum)");
    if (rc) return rc;
    GISAPR_CHECK_CUDA(launch_project_templates_planes((cudaStream_t)stream, (const float2*)spectrum, rot, dirs,
                                                      n_build, out_slot, mask, fsc, bt.list, bt.ptr, bt.count,
                                                      bt.n_bins, ctx->tw, ctx->tw3, (float2*)bank,
                                                      (float2*)ctx->proj_scratch.ptr, grid, box, newbox,
                                                      (float2*)ctx->proj_slices.ptr, (float2*)ctx->proj_blocked.ptr,
                                                      chunk),
                      "project_templates");
    ctx->blocked_box = box;
    return GISAPR_OK;
  }
  GISAPR_CHECK_CUDA(launch_project_templates((cudaStream_t)stream, (const float2*)spectrum, rot, dirs, n_build,
                                             out_slot, mask, fsc, bt.list, bt.ptr, bt.count, bt.n_bins,
                                             ctx->tw, ctx->tw3, (float2*)bank, (float2*)ctx->proj_scratch.ptr, grid,
                                             box, newbox),
                    "project_templates");
  return GISAPR_OK;
}

int gisapr_packed_ctf(void* stream, const float* dfu, const float* dfv, const float* dfa, int n,
                      const float* tx, const float* ty, const float* tu4, const float* tnc, int K,
                      float k1, float k2, float k3, float k5, float kk, float* out) {
  if (n < 0 || K <= 0) return fail(GISAPR_ERR_ARGUMENT, "n < 0 or K <= 0");
  if (n > 0 && (!dfu || !dfv || !dfa || !tx || !ty || !tu4 || !tnc || !out))
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (n > 65535) return fail(GISAPR_ERR_ARGUMENT, "at most 65535 particles per CTF call");
  GISAPR_CHECK_CUDA(launch_packed_ctf((cudaStream_t)stream, dfu, dfv, dfa, n, tx, ty, tu4, tnc, K, k1, k2,
                                      k3, k5, kk, out),
                    "packed_ctf");
  return GISAPR_OK;
}

int gisapr_prepare_particles(gisapr_ctx ctx, void* stream, const float* images, int n, int n_psi,
                             const int* psi_index, const float* psi_table, const float* mask,
                             const float* ctf, int box, int newbox, float* out) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n < 0 || n_psi <= 0) return fail(GISAPR_ERR_ARGUMENT, "n < 0 or n_psi <= 0");
  if (n > 0 && (!images || !psi_index || !psi_table || !ctf || !out))
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  int rc = check_box(box);
  if (rc) return rc;
  rc = check_newbox(box, newbox);
  if (rc) return rc;
  if (n == 0) return GISAPR_OK;
  rc = set_device(ctx);
  if (rc) return rc;
  const int grid = grid_for(ctx, n * n_psi, 4);
  rc = ensure(ctx, ctx->prep_scratch, (size_t)grid * prepare_scratch_elems(box, newbox) * sizeof(float2),
              "cudaMalloc(particle scratch)");
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_prepare_particles((cudaStream_t)stream, images, n, n_psi, psi_index, psi_table, mask,
                                             ctf, (float2*)out, (float2*)ctx->prep_scratch.ptr, grid, ctx->tw, ctx->tw3,
                                             box, newbox),
                    "prepare_particles");
  return GISAPR_OK;
}

int gisapr_correlate_batch_subset(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride,
                                  int n_cand, const float* stack, const int* local_ptr, const int* local_idx,
                                  int n_particles, int nnz, int n_psi, int n, int crop, const unsigned char* subset,
                                  float* out_score, int* out_y, int* out_x) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n_particles < 0 || n_psi <= 0 || n_cand < 0)
    return fail(GISAPR_ERR_ARGUMENT, "n_particles < 0, n_psi <= 0 or n_cand < 0");
  if (n_particles == 0 || n_cand == 0) return GISAPR_OK;
  if (!bank || !stack || !local_ptr || !local_idx || !out_score || !out_y || !out_x)
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (n_cand > 1 && bank_stride <= 0) return fail(GISAPR_ERR_ARGUMENT, "bank_stride must be positive");
  if (n < 32 || n > 256 || n % 16 != 0)
    return fail(GISAPR_ERR_UNSUPPORTED, "correlation size must be a multiple of 16 in [32, 256]");
  if (crop < 2 || crop > 16 || crop % 2 != 0 || crop > n)
    return fail(GISAPR_ERR_UNSUPPORTED, "crop must be even, 2..16 and <= n");
  const int cluster = tuned_cluster(ctx, n);
  const size_t smem = correlate_smem_bytes(n, n_psi, crop, cluster);
  if (smem > 227 * 1024)
    return fail(GISAPR_ERR_UNSUPPORTED, "too many psi angles for the shared-memory particle slice");
  int rc = set_device(ctx);
  if (rc) return rc;
  CorrTables t;
  rc = get_corr_tables(ctx, n, crop, &t);
  if (rc) return rc;
  if (nnz < 0) return fail(GISAPR_ERR_ARGUMENT, "nnz < 0");
  GISAPR_CHECK_CUDA(launch_correlate_plain((cudaStream_t)stream, (const float2*)bank, (const float2*)stack,
                                           local_ptr, local_idx, n_particles, n_psi, n, crop, t.outer, t.col,
                                           out_score, out_y, out_x, n_cand, bank_stride, nnz, cluster, subset),
                    "correlate");
  return GISAPR_OK;
}

int gisapr_correlate_batch(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride, int n_cand,
                           const float* stack, const int* local_ptr, const int* local_idx, int n_particles,
                           int nnz, int n_psi, int n, int crop, float* out_score, int* out_y, int* out_x) {
  return gisapr_correlate_batch_subset(ctx, stream, bank, bank_stride, n_cand, stack, local_ptr, local_idx,
                                       n_particles, nnz, n_psi, n, crop, nullptr, out_score, out_y, out_x);
}

int gisapr_correlate(gisapr_ctx ctx, void* stream, const float* bank, const float* stack,
                     const int* local_ptr, const int* local_idx, int n_particles, int n_psi, int n,
                     int crop, float* out_score, int* out_y, int* out_x) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n_particles < 0 || n_psi <= 0) return fail(GISAPR_ERR_ARGUMENT, "n_particles < 0 or n_psi <= 0");
  if (n_particles == 0) return GISAPR_OK;
  if (!bank || !stack || !local_ptr || !local_idx || !out_score || !out_y || !out_x)
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (n < 32 || n > 256 || n % 16 != 0)
    return fail(GISAPR_ERR_UNSUPPORTED, "correlation size must be a multiple of 16 in [32, 256]");
  if (crop < 2 || crop > 16 || crop % 2 != 0 || crop > n)
    return fail(GISAPR_ERR_UNSUPPORTED, "crop must be even, 2..16 and <= n");
  const int cluster = tuned_cluster(ctx, n);
  const size_t smem = correlate_smem_bytes(n, n_psi, crop, cluster);
  if (smem > 227 * 1024)
    return fail(GISAPR_ERR_UNSUPPORTED, "too many psi angles for the shared-memory particle slice");
  int rc = set_device(ctx);
  if (rc) return rc;
  CorrTables t;
  rc = get_corr_tables(ctx, n, crop, &t);
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_correlate_plain((cudaStream_t)stream, (const float2*)bank, (const float2*)stack,
                                           local_ptr, local_idx, n_particles, n_psi, n, crop, t.outer, t.col,
                                           out_score, out_y, out_x, 1, 0, 0, cluster, nullptr),
                    "correlate");
  return GISAPR_OK;
}

static int tuned(const std::map<int, int>& m, int n) {
  auto it = m.find(n);
  return it == m.end() ? 0 : it->second;
}

int gisapr_set_tuning(gisapr_ctx ctx, int key, int size, int value) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  switch (key) {
    case GISAPR_TUNE_TC_A_STAGES:
    case GISAPR_TUNE_TC_B_STAGES: {
      const int hi = key == GISAPR_TUNE_TC_A_STAGES ? 8 : 3;
      if (value != 0 && (value < 2 || value > hi))
        return fail(GISAPR_ERR_ARGUMENT, "ring depth must be 0 (default) or 2.." + std::to_string(hi));
      if (size != 32 && size != 64 && size != 96 && size != 128 && size != 192 && size != 256)
        return fail(GISAPR_ERR_ARGUMENT, "tensor-core correlation size must be one of 32, 64, 96, 128, 192, 256");
      auto& m = key == GISAPR_TUNE_TC_A_STAGES ? ctx->tune_tc_a : ctx->tune_tc_b;
      if (value == 0) m.erase(size);
      else m[size] = value;
      return GISAPR_OK;
    }
    case GISAPR_TUNE_CORR_CLUSTER:
      if (value < 0 || value > 8) return fail(GISAPR_ERR_ARGUMENT, "correlation cluster size must be 0..8");
      if (size < 32 || size > 256 || size % 16 != 0)
        return fail(GISAPR_ERR_ARGUMENT, "correlation size must be a multiple of 16 in [32, 256]");
      if (value == 0) ctx->tune_corr_cluster.erase(size);
      else ctx->tune_corr_cluster[size] = value;
      return GISAPR_OK;
    default:
      return fail(GISAPR_ERR_ARGUMENT, "unknown tuning key " + std::to_string(key));
  }
}

int gisapr_get_tuning(gisapr_ctx ctx, int key, int size, int* value) {
  if (!ctx || !value) return fail(GISAPR_ERR_ARGUMENT, "context or value is NULL");
  switch (key) {
    case GISAPR_TUNE_CORR_CLUSTER:
      *value = tuned(ctx->tune_corr_cluster, size);
      return GISAPR_OK;
    case GISAPR_TUNE_TC_A_STAGES:
      *value = tuned(ctx->tune_tc_a, size);
      return GISAPR_OK;
    case GISAPR_TUNE_TC_B_STAGES:
      *value = tuned(ctx->tune_tc_b, size);
      return GISAPR_OK;
    default:
      return fail(GISAPR_ERR_ARGUMENT, "unknown tuning key " + std::to_string(key));
  }
}

long long gisapr_tc_bank_bytes(int n_slot, int n) {
  if (n_slot < 0 || n <= 0) return 0;
  return correlate_tc_bank_halves(n_slot, n) * 2;
}

int gisapr_tc_plan_work(const int* local_ptr, const int* local_idx, int n_particles, int n_cand, int n_psi,
                        int crop, int* work, int max_work, int* n_work) {
  if (!n_work) return fail(GISAPR_ERR_ARGUMENT, "n_work is NULL");
  *n_work = 0;
  if (n_particles < 0 || n_cand <= 0 || n_psi <= 0)
    return fail(GISAPR_ERR_ARGUMENT, "n_particles < 0, n_cand <= 0 or n_psi <= 0");
  if (n_cand > correlate_tc_max_cand())
    return fail(GISAPR_ERR_ARGUMENT, "at most 128 candidates per tensor-core call");
  if (n_particles == 0) return GISAPR_OK;
  if (!local_ptr || !local_idx) return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  for (int b = 0; b < n_particles; ++b)
    if (local_ptr[b + 1] < local_ptr[b]) return fail(GISAPR_ERR_ARGUMENT, "local_ptr must be non-decreasing");
  if (crop < 2 || crop > 14 || crop % 2 != 0)
    return fail(GISAPR_ERR_UNSUPPORTED, "tensor-core correlation takes an even crop in 2..14");
  const int count = correlate_tc_plan(local_ptr, local_idx, n_particles, n_cand, n_psi, crop, nullptr, 0);
  if (work != nullptr) {
    if (max_work < count) return fail(GISAPR_ERR_ARGUMENT, "work holds fewer than the planned items");
    correlate_tc_plan(local_ptr, local_idx, n_particles, n_cand, n_psi, crop, work, max_work);
  }
  *n_work = count;
  return GISAPR_OK;
}

int gisapr_correlate_tc_batch_ex(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride,
                                 int n_cand, int n_slot, void* tbank, const float* stack, const int* local_ptr,
                                 const int* local_idx, const int* work, int n_work, int nnz, int n_psi, int n,
                                 int crop, int precision, const float* col_scale_t, const float* col_scale_p,
                                 unsigned wait_limit, float* out_score, int* out_y, int* out_x, int* status) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n_cand < 0 || n_slot < 0 || n_work < 0 || nnz < 0 || n_psi <= 0)
    return fail(GISAPR_ERR_ARGUMENT, "n_cand, n_slot, n_work or nnz < 0, or n_psi <= 0");
  if (precision < GISAPR_TC_FP16 || precision > GISAPR_TC_BF16X3)
    return fail(GISAPR_ERR_ARGUMENT, "precision must be GISAPR_TC_FP16, _FP16X3, _BF16 or _BF16X3");
  if (n_cand == 0 || n_work == 0) return GISAPR_OK;
  if (!bank || !tbank || !stack || !local_ptr || !local_idx || !work || !out_score || !out_y || !out_x)
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (n_slot == 0) return fail(GISAPR_ERR_ARGUMENT, "n_slot must be positive when there is work");
  if (n_cand > 1 && bank_stride < (long long)n_slot * n * (n / 2 + 1))
    return fail(GISAPR_ERR_ARGUMENT, "bank_stride is smaller than one candidate's bank");
  if (n != 32 && n != 64 && n != 96 && n != 128 && n != 192 && n != 256)
    return fail(GISAPR_ERR_UNSUPPORTED, "tensor-core correlation takes n in {32, 64, 96, 128, 192, 256}");
  if (crop < 2 || crop > 14 || crop % 2 != 0 || crop > n || (n == 256 && crop < 10))
    return fail(GISAPR_ERR_UNSUPPORTED, "tensor-core correlation takes an even crop in 2..14 (10..14 at n = 256)");
  if (n_slot > 65535) return fail(GISAPR_ERR_ARGUMENT, "at most 65535 template slots");
  if (n_cand > correlate_tc_max_cand())
    return fail(GISAPR_ERR_ARGUMENT, "at most 128 candidates per tensor-core call");
  if (((uintptr_t)tbank & 15) != 0) return fail(GISAPR_ERR_ARGUMENT, "tbank must be 16-byte aligned");
  int rc = set_device(ctx);
  if (rc) return rc;
  CorrTables t;
  rc = get_corr_tables(ctx, n, crop, &t);
  if (rc) return rc;
  const cudaStream_t st = (cudaStream_t)stream;
  const int bf16 = (precision == GISAPR_TC_BF16 || precision == GISAPR_TC_BF16X3) ? 1 : 0;
  const int split = (precision == GISAPR_TC_FP16X3 || precision == GISAPR_TC_BF16X3) ? 1 : 0;
  GISAPR_CHECK_CUDA(launch_bank_to_operands(st, (const float2*)bank, bank_stride, n_cand, n_slot, n, bf16, split,
                                            col_scale_t, tbank, status),
                    "bank_to_operands");
  const int grid = std::min(n_work, ctx->sm_count);
  GISAPR_CHECK_CUDA(launch_correlate_tc(st, tbank, n_cand, (const float2*)stack, local_ptr, local_idx, work, n_work,
                                        n_psi, n, crop, nnz, split, bf16, col_scale_t, col_scale_p, wait_limit,
                                        t.row, t.col, out_score, out_y, out_x, status, grid,
                                        tuned(ctx->tune_tc_a, n), tuned(ctx->tune_tc_b, n)),
                    "correlate_tc");
  return GISAPR_OK;
}

int gisapr_correlate_tc_batch(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride, int n_cand,
                              int n_slot, void* tbank, const float* stack, const int* local_ptr,
                              const int* local_idx, const int* work, int n_work, int nnz, int n_psi, int n, int crop,
                              int split, float* out_score, int* out_y, int* out_x, int* status) {
  return gisapr_correlate_tc_batch_ex(ctx, stream, bank, bank_stride, n_cand, n_slot, tbank, stack, local_ptr,
                                      local_idx, work, n_work, nnz, n_psi, n, crop,
                                      split ? GISAPR_TC_FP16X3 : GISAPR_TC_FP16, nullptr, nullptr, 0, out_score, out_y,
                                      out_x, status);
}

int gisapr_particle_results_subset(void* stream, const int* local_ptr, const float* score, const int* ys,
                                   const int* xs, int n_particles, int n_psi, int n_cand,
                                   const unsigned char* subset, int* best_entry, int* best_psi, float* peak,
                                   int* peak_y, int* peak_x, float* zscore) {
  if (n_particles < 0 || n_psi <= 0 || n_cand < 0)
    return fail(GISAPR_ERR_ARGUMENT, "n_particles < 0, n_psi <= 0 or n_cand < 0");
  if (n_particles == 0 || n_cand == 0) return GISAPR_OK;
  if (!local_ptr || !score || !ys || !xs || !best_entry || !best_psi || !peak || !peak_y || !peak_x ||
      !zscore)
    return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (n_cand > 65535) return fail(GISAPR_ERR_ARGUMENT, "at most 65535 candidates per call");
  GISAPR_CHECK_CUDA(launch_particle_results((cudaStream_t)stream, local_ptr, score, ys, xs, n_particles, n_psi,
                                            best_entry, best_psi, peak, peak_y, peak_x, zscore, n_cand, subset),
                    "particle_results");
  return GISAPR_OK;
}

int gisapr_particle_results_batch(void* stream, const int* local_ptr, const float* score, const int* ys,
                                  const int* xs, int n_particles, int n_psi, int n_cand, int* best_entry,
                                  int* best_psi, float* peak, int* peak_y, int* peak_x, float* zscore) {
  return gisapr_particle_results_subset(stream, local_ptr, score, ys, xs, n_particles, n_psi, n_cand, nullptr,
                                        best_entry, best_psi, peak, peak_y, peak_x, zscore);
}

int gisapr_particle_results(void* stream, const int* local_ptr, const float* score, const int* ys,
                            const int* xs, int n_particles, int n_psi, int* best_entry, int* best_psi,
                            float* peak, int* peak_y, int* peak_x, float* zscore) {
  return gisapr_particle_results_batch(stream, local_ptr, score, ys, xs, n_particles, n_psi, 1, best_entry,
                                       best_psi, peak, peak_y, peak_x, zscore);
}

int gisapr_score_sum_subset(void* stream, const int* local_ptr, const float* peak, int n_particles, int n_cand,
                            const unsigned char* subset, double* out) {
  if (n_particles < 0 || n_cand < 0 || !out) return fail(GISAPR_ERR_ARGUMENT, "bad arguments");
  if (n_particles > 0 && (!local_ptr || !peak)) return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  GISAPR_CHECK_CUDA(launch_score_sum((cudaStream_t)stream, local_ptr, peak, n_particles, out, n_cand, subset),
                    "score_sum");
  return GISAPR_OK;
}

int gisapr_score_sum_batch(void* stream, const int* local_ptr, const float* peak, int n_particles, int n_cand,
                           double* out) {
  return gisapr_score_sum_subset(stream, local_ptr, peak, n_particles, n_cand, nullptr, out);
}

int gisapr_score_sum(void* stream, const int* local_ptr, const float* peak, int n_particles, double* out) {
  return gisapr_score_sum_batch(stream, local_ptr, peak, n_particles, 1, out);
}

int gisapr_ingest_stack(gisapr_ctx ctx, void* stream, const float* images, int n, int h, int w, const int* shifts,
                        int ch, int cw, int flags, const int* bin_ptr, const int* bin_pix, const double* bin_count,
                        int n_bins, const double* highpass_mask, double* work, float* out) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (n < 0 || h < 1 || w < 1) return fail(GISAPR_ERR_ARGUMENT, "n < 0 or an image side < 1");
  if (ch < 1 || cw < 1 || ch > h || cw > w)
    return fail(GISAPR_ERR_ARGUMENT, "the crop must be at least 1 and at most the image size on both axes");
  if (flags & ~7) return fail(GISAPR_ERR_ARGUMENT, "unknown flag bits");
  if ((flags & 1) && (!bin_ptr || !bin_pix || !bin_count || n_bins < 1 || n_bins > 8192))
    return fail(GISAPR_ERR_ARGUMENT, "whitening needs the radial bin tables (1..8192 bins)");
  if ((flags & 4) && !highpass_mask) return fail(GISAPR_ERR_ARGUMENT, "the high-pass mask is NULL");
  if (n == 0) return GISAPR_OK;
  if (!images || !work || !out) return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if ((long long)ch * cw > (1LL << 26)) return fail(GISAPR_ERR_ARGUMENT, "crop too large");
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int pixels = ch * cw;
  double2* wk = (double2*)work;
  GISAPR_CHECK_CUDA(launch_ingest_load(st, images, n, h, w, shifts, ch, cw, wk, ctx->sm_count), "ingest_load");
  cufftHandle plan = 0;
  if (flags & 5) {
    int dims[2] = {ch, cw};
    cufftResult r = cufftPlanMany(&plan, 2, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_Z2Z, n);
    if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftPlanMany(Z2Z) failed with code " + std::to_string((int)r));
    cufftSetStream(plan, st);
  }
  auto run = [&]() -> int {
    const double inv = 1.0 / (double)pixels;
    double scale = 1.0;  // pending factor of the values in work
    if (flags & 1) {
      cufftResult r = cufftExecZ2Z(plan, (cufftDoubleComplex*)wk, (cufftDoubleComplex*)wk, CUFFT_FORWARD);
      if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftExecZ2Z failed");
      GISAPR_CHECK_CUDA(launch_ingest_spectrum_divide(st, wk, n, pixels, bin_ptr, bin_pix, bin_count, n_bins),
                        "ingest_spectrum_divide");
      r = cufftExecZ2Z(plan, (cufftDoubleComplex*)wk, (cufftDoubleComplex*)wk, CUFFT_INVERSE);
      if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftExecZ2Z failed");
      scale = inv;
    }
    if (flags & 2) {
      GISAPR_CHECK_CUDA(launch_ingest_normalize(st, wk, n, ch, cw, scale), "ingest_normalize");
      scale = 1.0;
    }
    if (flags & 4) {
      if (scale != 1.0)  // the real image of the preceding inverse transform
        GISAPR_CHECK_CUDA(launch_ingest_scale_mask(st, wk, n, pixels, nullptr, scale, 1, ctx->sm_count),
                          "ingest_scale");
      cufftResult r = cufftExecZ2Z(plan, (cufftDoubleComplex*)wk, (cufftDoubleComplex*)wk, CUFFT_FORWARD);
      if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftExecZ2Z failed");
      GISAPR_CHECK_CUDA(launch_ingest_scale_mask(st, wk, n, pixels, highpass_mask, 1.0, 0, ctx->sm_count),
                        "ingest_mask");
      r = cufftExecZ2Z(plan, (cufftDoubleComplex*)wk, (cufftDoubleComplex*)wk, CUFFT_INVERSE);
      if (r != CUFFT_SUCCESS) return fail(GISAPR_ERR_CUFFT, "cufftExecZ2Z failed");
      scale = inv;
    }
    GISAPR_CHECK_CUDA(launch_ingest_store(st, wk, n, pixels, scale, out, ctx->sm_count), "ingest_store");
    return GISAPR_OK;
  };
  rc = run();
  if (plan) {
    // the plan's work area may be in use until the stream reaches this point
    cudaStreamSynchronize(st);
    cufftDestroy(plan);
  }
  return rc;
}

int gisapr_restraint_edt(gisapr_ctx ctx, void* stream, const float* density, int box, float threshold,
                         unsigned char* mask, int* d2, int* scratch) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (!density || !mask || !d2 || !scratch) return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (box < 1 || box > 1024) return fail(GISAPR_ERR_ARGUMENT, "box must be in [1, 1024]");
  if (!std::isfinite(threshold)) return fail(GISAPR_ERR_ARGUMENT, "threshold must be finite");
  int rc = set_device(ctx);
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_restraint_edt((cudaStream_t)stream, density, threshold, mask, d2, scratch, box),
                    "restraint_edt");
  return GISAPR_OK;
}

int gisapr_restraint_init(void* stream, int* out, int n) {
  if (n < 0 || (n > 0 && !out)) return fail(GISAPR_ERR_ARGUMENT, "bad arguments");
  if (n == 0) return GISAPR_OK;
  GISAPR_CHECK_CUDA(launch_restraint_init((cudaStream_t)stream, out, n), "restraint_init");
  return GISAPR_OK;
}

int gisapr_restraint_eval(gisapr_ctx ctx, void* stream, float* volume, const unsigned char* mask, const int* d2,
                          int box, const int* bounds, float threshold, int* out) {
  if (!ctx) return fail(GISAPR_ERR_ARGUMENT, "context is NULL");
  if (!volume || !mask || !d2 || !bounds || !out) return fail(GISAPR_ERR_ARGUMENT, "a required pointer is NULL");
  if (box < 1 || box > 1024) return fail(GISAPR_ERR_ARGUMENT, "box must be in [1, 1024]");
  for (int a = 0; a < 3; ++a)
    if (bounds[a] < 0 || bounds[3 + a] > box || bounds[a] > bounds[3 + a])
      return fail(GISAPR_ERR_ARGUMENT, "bounds must satisfy 0 <= lo <= hi <= box on every axis");
  int rc = set_device(ctx);
  if (rc) return rc;
  GISAPR_CHECK_CUDA(launch_restraint_reduce((cudaStream_t)stream, volume, mask, d2, box, bounds, bounds + 3,
                                            threshold, out, ctx->sm_count),
                    "restraint_reduce");
  return GISAPR_OK;
}

}  // extern "C"
