// Fixed-footprint neighbour search: the same cell-list pair search as the
// domain's rebuild (reference cell index, radius rule rij / h <= Cellfac,
// canonical row order), for callers that cannot allocate device memory.
//
// Who needs this: code that runs where cudaMalloc is off limits — inside a
// host callback, inside another library's memory pool that owns every byte of
// the device, in a plugin host that forbids device allocations, or in a
// real-time loop where an allocation could stall or fail.  Such a caller owns
// its input and output buffers; the only working memory this search needs
// (cell histogram, cell offsets, cell-sorted particle list) lives in one
// file-scope device array below, reserved when the library is loaded and kept
// by every GPU that loads it until the process exits.
//
// Limits: at most WF_STATIC_MAX_PARTICLES particles and WF_STATIC_MAX_CELLS
// grid cells per call (about 10 MB of scratch per device).  Every call uses
// the same array, so calls whose work overlaps on the GPU (two streams, or
// two host threads) race and must be serialised by the caller.  The first call
// on a device looks up the array's device address (cudaGetSymbolAddress) with
// that device current; make that first call before any stream capture.  The
// look-up is repeated when the device's context has been destroyed and
// re-created since the last call (cudaDeviceReset), which reloads the array.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/weldform_gb300.h"

namespace wf {
void set_last_error(const std::string& msg);  // the message wf_last_error() returns
}

namespace {

constexpr long long kMaxParticles = WF_STATIC_MAX_PARTICLES;
constexpr long long kMaxCells = WF_STATIC_MAX_CELLS;
constexpr int kMaxNb = 100;  // neighbours per particle (MAX_NB_PER_PART, Source/Domain.h:49)

struct Scratch {
  int cell_count[kMaxCells];      // histogram, reused as scatter cursor
  int cell_start[kMaxCells + 1];  // exclusive prefix of the histogram
  int cell_of[kMaxParticles];     // cell of each particle
  int sorted[kMaxParticles];      // particle indices grouped by cell
};

// The working memory of wf_neighbour_list_static (see the file comment).
static __device__ __align__(256) unsigned char g_scratch[sizeof(Scratch)];

int fail(int code, const std::string& m) { wf::set_last_error(m); return code; }

struct Grid {
  double blpf[3], cs[3];
  int no[3];
  double cellfac;
};

__device__ __forceinline__ int cell_index(const Grid& g, double x, double y, double z) {
  double p[3] = {x, y, z};
  int c[3];
  for (int d = 0; d < 3; ++d) {
    int q = (int)floor(__ddiv_rn(__dsub_rn(p[d], g.blpf[d]), g.cs[d]));
    c[d] = q < 0 ? 0 : (q >= g.no[d] ? g.no[d] - 1 : q);
  }
  return (c[0] * g.no[1] + c[1]) * g.no[2] + c[2];
}

__global__ void k_static_clear(Scratch* s, int ncells) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncells; k += gridDim.x * blockDim.x) s->cell_count[k] = 0;
}

__global__ void k_static_hist(Scratch* s, Grid g, const double* x, const double* y, const double* z, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int c = cell_index(g, x[p], y[p], z[p]);
  s->cell_of[p] = c;
  atomicAdd(&s->cell_count[c], 1);
}

// Single-block exclusive scan: thread t owns a contiguous chunk of cells.
__global__ void k_static_scan(Scratch* s, int ncells) {
  __shared__ long long part[1024];
  int t = threadIdx.x;
  int chunk = (ncells + blockDim.x - 1) / blockDim.x;
  int b = t * chunk, e = min(ncells, b + chunk);
  long long sum = 0;
  for (int k = b; k < e; ++k) sum += s->cell_count[k];
  part[t] = sum;
  __syncthreads();
  if (t == 0) {
    long long run = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) { long long v = part[k]; part[k] = run; run += v; }
    s->cell_start[ncells] = (int)run;
  }
  __syncthreads();
  long long run = part[t];
  for (int k = b; k < e; ++k) { s->cell_start[k] = (int)run; run += s->cell_count[k]; s->cell_count[k] = 0; }
}

__global__ void k_static_scatter(Scratch* s, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int c = s->cell_of[p];
  s->sorted[s->cell_start[c] + atomicAdd(&s->cell_count[c], 1)] = p;
}

__global__ void __launch_bounds__(128) k_static_rows(Scratch* s, Grid g, const double* x, const double* y,
                                                     const double* z, const double* h, int n, int32_t* row_len,
                                                     int32_t* nbr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int row[kMaxNb];
  unsigned keys[kMaxNb];
  int cnt = 0;
  bool over = false;
  double xi = x[i], yi = y[i], zi = z[i], hi = h[i];
  int ci = cell_index(g, xi, yi, zi);
  int c0 = ci / (g.no[1] * g.no[2]), c1 = (ci / g.no[2]) % g.no[1], c2 = ci % g.no[2];
  for (int a = c0 - 1; a <= c0 + 1; ++a) {
    if (a < 0 || a >= g.no[0]) continue;
    for (int b = c1 - 1; b <= c1 + 1; ++b) {
      if (b < 0 || b >= g.no[1]) continue;
      for (int e = c2 - 1; e <= c2 + 1; ++e) {
        if (e < 0 || e >= g.no[2]) continue;
        int c = (a * g.no[1] + b) * g.no[2] + e;
        for (int k = s->cell_start[c]; k < s->cell_start[c + 1]; ++k) {
          int j = s->sorted[k];
          if (j == i) continue;
          // CheckRadius (Neighbour.cpp:361-372), IEEE operations, no contraction.
          double hh = __ddiv_rn(__dadd_rn(hi, h[j]), 2.0);
          double dx = __dsub_rn(xi, x[j]), dy = __dsub_rn(yi, y[j]), dz = __dsub_rn(zi, z[j]);
          double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
          if (!(__ddiv_rn(r, hh) <= g.cellfac)) continue;
          unsigned kk = (unsigned)(j - i - 1);  // j > i ascending, then j < i ascending
          // Sorted insertion that keeps the kMaxNb smallest keys: the row does
          // not depend on the order in which the cells list their particles.
          int m = cnt - 1;
          if (cnt == kMaxNb) {
            over = true;
            if (kk > keys[kMaxNb - 1]) continue;
            m = kMaxNb - 2;  // the largest key drops out
          } else {
            ++cnt;
          }
          while (m >= 0 && keys[m] > kk) { keys[m + 1] = keys[m]; row[m + 1] = row[m]; --m; }
          keys[m + 1] = kk;
          row[m + 1] = j;
        }
      }
    }
  }
  for (int k = 0; k < cnt; ++k) nbr[(size_t)k * n + i] = row[k];
  row_len[i] = over ? kMaxNb + 1 : cnt;  // 101: the row was cut at its 100 smallest keys
}

// The array's device address per device, with the identity of the context it
// was looked up in (cuCtxGetId, reached through the runtime's driver entry
// points so the library needs no link to the driver library).
std::mutex g_mu;
void* g_addr[64] = {nullptr};
unsigned long long g_ctx_id[64] = {0};

unsigned long long current_context_id() {
  typedef int (*GetCurrent)(void**);
  typedef int (*GetId)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;  // unknown: the cached address is kept
}

}  // namespace

extern "C" int wf_neighbour_list_static(const double* x, const double* y, const double* z, const double* h,
                                        int64_t n, const double blpf[3], const double cell_size[3],
                                        const int32_t cell_no[3], double cellfac, int32_t* row_len,
                                        int32_t* nbr, void* stream) {
  if (n < 0 || n > kMaxParticles)
    return fail(WF_ERR_ARG, "wf_neighbour_list_static: n = " + std::to_string(n) + " exceeds the fixed maximum of " +
                                std::to_string(kMaxParticles) + " particles");
  if (!x || !y || !z || !h || !row_len || !nbr || !blpf || !cell_size || !cell_no)
    return fail(WF_ERR_ARG, "wf_neighbour_list_static: null pointer argument");
  long long ncells = 1;
  for (int d = 0; d < 3; ++d) {
    if (cell_no[d] <= 0 || !(cell_size[d] > 0)) return fail(WF_ERR_ARG, "wf_neighbour_list_static: empty cell grid");
    if (cell_no[d] > kMaxCells / ncells)  // checked before the product can overflow
      return fail(WF_ERR_ARG, "wf_neighbour_list_static: the cell grid " + std::to_string(cell_no[0]) + " x " +
                                  std::to_string(cell_no[1]) + " x " + std::to_string(cell_no[2]) +
                                  " exceeds the fixed maximum of " + std::to_string(kMaxCells) + " cells");
    ncells *= cell_no[d];
  }
  if (n == 0) return WF_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(WF_ERR_CUDA, "wf_neighbour_list_static: no current CUDA device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long ctx = current_context_id();
    // set-up on the first call on this device, and again in a re-created
    // context (keep the first call outside stream capture)
    if (!g_addr[dev] || (ctx != 0 && ctx != g_ctx_id[dev])) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess)
        return fail(WF_ERR_CUDA, std::string("wf_neighbour_list_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_addr[dev] = p;
      g_ctx_id[dev] = ctx;
    }
    base = g_addr[dev];
  }
  Scratch* s = static_cast<Scratch*>(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Grid g;
  for (int d = 0; d < 3; ++d) { g.blpf[d] = blpf[d]; g.cs[d] = cell_size[d]; g.no[d] = cell_no[d]; }
  g.cellfac = cellfac;
  int nn = (int)n, nc = (int)ncells;
  k_static_clear<<<256, 256, 0, st>>>(s, nc);
  k_static_hist<<<(nn + 255) / 256, 256, 0, st>>>(s, g, x, y, z, nn);
  k_static_scan<<<1, 1024, 0, st>>>(s, nc);
  k_static_scatter<<<(nn + 255) / 256, 256, 0, st>>>(s, nn);
  k_static_rows<<<(nn + 127) / 128, 128, 0, st>>>(s, g, x, y, z, h, nn, row_len, nbr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WF_ERR_CUDA, std::string("wf_neighbour_list_static: ") + cudaGetErrorString(e));
  return WF_OK;
}

