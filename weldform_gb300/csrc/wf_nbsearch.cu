// Neighbour search of the kick-drift step on sm_103a.
//
// Replaces the reference's linked-list cell search (Neighbour.cpp:10-477) and
// pair-list flattening (CalcPairPosList, Neighbour.cpp:617-694):
//   1. k_cell_keys   — reference cell index (ListGenerate, Neighbour.cpp:183-227:
//                      floor((x - BLPF) / CellSize), clamped) mapped to the cell's
//                      Morton rank; histogram per cell.
//   2. exclusive scan of the histogram -> cell start offsets.
//   3. k_scatter + k_sort_cells — counting-sort scatter, then each cell's slots
//                      ordered by original particle index (deterministic order).
//   4. k_permute / k_copy_back — every persistent state column reordered.
//   5. k_nbr_fill    — one warp per particle scans the 27 neighbouring cells,
//                      applies the reference pair rules (AllocateNbPair,
//                      Neighbour.cpp:374-417: contact-surface pairs, radius test
//                      CheckRadius :361-372, free + same material) and writes its
//                      row in canonical order (j > i ascending, then j < i
//                      ascending by original index) into an ELL array
//                      (entry k of particle i at k * N + i).
// With the Verlet-skin reuse, a full search (steps 1-5) also builds each
// particle's superset over a 5 x 5 x 5 stencil at the pair radius plus the
// skin (k_nbr_fill<true>), and a later search whose particles all moved less
// than half the skin skips steps 1-5 and filters the supersets with the same
// exact rules (k_skin_check, k_search_mode, k_cell_coords, k_nbr_filter).
// The radius test rij / h <= Cellfac is decided bit-exactly: an FP32 distance
// prefilter with a proven-safe relative margin accepts or rejects clear cases,
// and everything inside the margin is decided by the reference's FP64
// expression evaluated with non-contracted IEEE operations.
//
// Every kernel checks st->do_search first (the re-sorting ones also
// search_full), so the search can sit inside a captured step and cost only
// an empty launch on steps that do not rebuild.
#include "wf_device.cuh"
#include "wf_launch.h"

namespace wf {

__device__ __forceinline__ bool searching(const DevPtrs& P) { return P.st->do_search != 0; }
// The parts of a search that re-sort the particles run only when the search
// is a full one (always, unless the Verlet-skin reuse is on).
__device__ __forceinline__ bool searching_full(const DevPtrs& P) {
  return P.st->do_search != 0 && P.st->search_full != 0;
}

// A particle with a non-finite coordinate cannot pass CheckRadius with any
// other (its distance is NaN or infinite), so its row is empty and it is in
// no other row.  The reference bins it into a clamped edge cell
// (Neighbour.cpp:185-218), where every later search scans all such particles
// pairwise.  Here it goes to one of ncells shadow buckets after the grid's
// (key ncells + original index mod ncells), which no stencil visits: the rows
// are the same and the search stays linear.  The shadow buckets are sorted
// like cells, so the order stays deterministic.
__global__ void k_cell_keys(DevPtrs P, DomainConst K) {
  if (!searching_full(P)) return;
  int nonfinite = 0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
  int c[3];
  bool finite = true;
  for (int d = 0; d < 3; ++d) {
    double xd = P.f[(C_X + d) * (size_t)K.N + p];
    finite = finite && isfinite(xd);
    int q = (int)floor(__ddiv_rn(__dsub_rn(xd, K.BLPF[d]), K.CellSize[d]));
    if (q < 0) q = 0;
    if (q >= K.CellNo[d]) q = K.CellNo[d] - 1;
    c[d] = q;
  }
  int key;
  if (finite) {
    key = P.cell_rank[(c[0] * K.CellNo[1] + c[1]) * K.CellNo[2] + c[2]];
  } else {
    key = K.ncells + P.i[I_ORIG * (size_t)K.N + p] % K.ncells;
    ++nonfinite;
  }
  P.i[I_CELL * (size_t)K.N + p] = key;
  atomicAdd(&P.cell_count[key], 1);
  }
  if (nonfinite) {
    atomicAdd(&P.st->nan_count, nonfinite);
    if (K.nan_check) atomicOr(&P.st->errors, ERR_NAN);
  }
}

// Batched domain, before the reordering (a full search): the rows of
// particles whose specimen does not search this step are saved by old
// position, each entry as the neighbour's original index (with the
// larger-index bit), so k_nbr_fill can put them back at the particles' new
// positions.
__global__ void k_rows_save(DevPtrs P, DomainConst K) {
  if (!searching_full(P)) return;
  const size_t N = K.N;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
    if (P.sp[P.i[I_SPEC * N + p]].do_search) continue;
    int len = P.row_len[p];
    P.save_len[p] = len;
    for (int k = 0; k < len; ++k) {
      int e = P.nbr[(size_t)k * N + p];
      P.save_nbr[(size_t)k * N + p] = P.i[I_ORIG * N + nb_index(e)] | (int)((unsigned)e & NB_UP);
    }
  }
}

__global__ void k_zero_int(DevPtrs P, int* a, long long n, int gate) {
  if (gate && !searching_full(P)) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) a[k] = 0;
}

// ---- exclusive scan of an int array into an int array (three phases) ------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* sh, long long* total) {
  // Hillis-Steele over a power-of-two block; deterministic.
  int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    long long add = (t >= off) ? sh[t - off] : 0;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  long long incl = sh[t];
  *total = sh[blockDim.x - 1];
  __syncthreads();
  return incl - v;
}

__global__ void k_scan_reduce(DevPtrs P, const int* in, long long n, long long* tot) {
  if (!searching_full(P)) return;
  __shared__ long long sh[SCAN_THREADS];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  long long s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long idx = base + (long long)threadIdx.x * SCAN_ITEMS + k;
    if (idx < n) s += in[idx];
  }
  long long total;
  block_exclusive_scan(s, sh, &total);
  if (threadIdx.x == 0) tot[blockIdx.x] = total;
}
__global__ void k_scan_top(DevPtrs P, long long* tot, int nb) {
  if (!searching_full(P)) return;
  __shared__ long long sh[SCAN_THREADS];
  long long carry = 0;
  for (int base = 0; base < nb; base += SCAN_THREADS) {
    int idx = base + threadIdx.x;
    long long v = (idx < nb) ? tot[idx] : 0;
    long long total;
    long long ex = block_exclusive_scan(v, sh, &total);
    if (idx < nb) tot[idx] = ex + carry;
    carry += total;
    __syncthreads();
  }
}
__global__ void k_scan_down(DevPtrs P, const int* in, long long n, const long long* tot, int* out, int* total_out) {
  if (!searching_full(P)) return;
  __shared__ long long sh[SCAN_THREADS];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  long long vals[SCAN_ITEMS];
  long long s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long idx = base + (long long)threadIdx.x * SCAN_ITEMS + k;
    vals[k] = (idx < n) ? in[idx] : 0;
    s += vals[k];
  }
  long long total;
  long long ex = block_exclusive_scan(s, sh, &total) + tot[blockIdx.x];
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long idx = base + (long long)threadIdx.x * SCAN_ITEMS + k;
    if (idx < n) out[idx] = (int)ex;
    ex += vals[k];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *total_out = (int)ex;
}

__global__ void k_scatter(DevPtrs P, DomainConst K) {
  if (!searching_full(P)) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
  int key = P.i[I_CELL * (size_t)K.N + p];
  int pos = P.cell_start[key] + atomicAdd(&P.cell_count[key], 1);
  P.perm[pos] = p;
  }
}

// Order each cell's slots by original particle index (insertion sort; cells
// hold ~10-20 particles), and likewise the shadow buckets of non-finite
// particles (at most ceil(N / ncells) each).
__global__ void k_sort_cells(DevPtrs P, DomainConst K) {
  if (!searching_full(P)) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < 2 * K.ncells; c += gridDim.x * blockDim.x) {
  int b = P.cell_start[c], e = P.cell_start[c + 1];
  const int* orig = P.i + I_ORIG * (size_t)K.N;
  for (int k = b + 1; k < e; ++k) {
    int v = P.perm[k];
    int ov = orig[v];
    int m = k - 1;
    while (m >= b && orig[P.perm[m]] > ov) { P.perm[m + 1] = P.perm[m]; --m; }
    P.perm[m + 1] = v;
  }
  }
}

// Gather every persistent column into the scratch arenas (new order).  A
// fixed grid strides over (column, particle) so the launch costs nothing on
// steps that do not search.
__global__ void k_permute(DevPtrs P, DomainConst K, double* fdst, int* idst) {
  if (!searching_full(P)) return;
  size_t N = K.N;
  size_t total = (size_t)(NF64_PERSIST + NI32_PERSIST) * N;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    size_t col = k / N, p = k - col * N;
    int src = P.perm[p];
    if (col < (size_t)NF64_PERSIST) fdst[col * N + p] = P.f[col * N + src];
    else {
      size_t c = col - NF64_PERSIST;
      idst[c * N + p] = P.i[c * N + src];
    }
  }
}
__global__ void k_copy_back(DevPtrs P, DomainConst K, const double* fsrc, const int* isrc) {
  if (!searching_full(P)) return;
  size_t nf = (size_t)NF64_PERSIST * K.N, ni = (size_t)NI32_PERSIST * K.N;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < nf + ni; k += (size_t)gridDim.x * blockDim.x) {
    if (k < nf) P.f[k] = fsrc[k];
    else P.i[k - nf] = isrc[k - nf];
  }
}

__device__ __forceinline__ bool is_contact_id(const DomainConst& K, int id) {
  for (int m = 0; m < K.nmeshes; ++m)
    if (id == K.contact_surf_id[m]) return true;
  return false;
}

// Map original -> sorted index, element -> mesh particle, and the FP32
// prefilter coordinates (relative to BLPF, plus h).
__global__ void k_after_permute(DevPtrs P, DomainConst K) {
  if (!searching_full(P)) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
  size_t N = K.N;
  int o = P.i[I_ORIG * N + p];
  P.inv[o] = p;
  int kind = P.i[I_KIND * N + p];
  if (kind == 1) P.elem_particle[P.i[I_ELEM * N + p]] = p;
  reinterpret_cast<float4*>(P.xs)[p] =
      make_float4((float)(P.f[(C_X + 0) * N + p] - K.BLPF[0]), (float)(P.f[(C_X + 1) * N + p] - K.BLPF[1]),
                  (float)(P.f[(C_X + 2) * N + p] - K.BLPF[2]), (float)P.f[C_H * N + p]);
  // class word for the pair rules: bit 0 rigid-mesh particle, bit 1 carries a
  // contact-surface id, bits 2.. material index
  P.i[I_CLASS * N + p] = kind | (is_contact_id(K, P.i[I_ID * N + p]) ? 2 : 0) | (P.i[I_MATERIAL * N + p] << 2);
  }
}


// CheckRadius (Neighbour.cpp:361-372) exactly: rij / ((hi + hj) / 2) <= Cellfac
// with rij = sqrt(dx*dx + dy*dy + dz*dz) summed left to right, no contraction.
__device__ __forceinline__ bool radius_exact(const DevPtrs& P, size_t N, int i, int j, double Cellfac) {
  double hh = __ddiv_rn(__dadd_rn(P.f[C_H * N + i], P.f[C_H * N + j]), 2.0);
  double dx = __dsub_rn(P.f[(C_X + 0) * N + i], P.f[(C_X + 0) * N + j]);
  double dy = __dsub_rn(P.f[(C_X + 1) * N + i], P.f[(C_X + 1) * N + j]);
  double dz = __dsub_rn(P.f[(C_X + 2) * N + i], P.f[(C_X + 2) * N + j]);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  double rij = __dsqrt_rn(s);
  return __ddiv_rn(rij, hh) <= Cellfac;
}

// Radius test: FP32 prefilter, exact FP64 decision inside the margin.
__device__ __forceinline__ bool radius_ok(const DevPtrs& P, const DomainConst& K, size_t N, int i, int j, float xi,
                                          float yi, float zi, float hi, float4 pj) {
  float dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  float R = K.half_cellfac_f * (hi + pj.w);
  float R2 = R * R;
  if (d2 < R2 * (1.0f - K.pre_eps)) return true;
  if (d2 > R2 * (1.0f + K.pre_eps)) return false;
  return radius_exact(P, N, i, j, K.Cellfac);
}

// SM neighbour rows in canonical order: one warp per particle, 32 consecutive
// particles per block.  Lanes test the candidates of each of the 27 cells in
// parallel; accepted ones are compacted with a ballot into the warp's shared
// buffer (128 slots), placed there by the rank of their canonical key, and the
// block writes its 32 rows to the ELL array one coalesced line per entry
// index.  Also sets Nb and the "free surface at search time" flag used by the
// contact pair rule.
// rank[r] += number of keys in row[0, n4) below key[r], r < NK (n4 a multiple of 4).
template <int NK>
__device__ __forceinline__ void rank_row(const unsigned* row, int n4, const unsigned key[4], int rank[4]) {
  for (int t = 0; t < n4; t += 4) {
    uint4 q = *reinterpret_cast<const uint4*>(row + t);
#pragma unroll
    for (int r = 0; r < NK; ++r)
      rank[r] += (int)(q.x < key[r]) + (int)(q.y < key[r]) + (int)(q.z < key[r]) + (int)(q.w < key[r]);
  }
}

constexpr int FILL_WARPS = 8;                    // warps per block
constexpr int FILL_ROWS = 32;                    // particles (rows) per block group
constexpr int FILL_PER_WARP = FILL_ROWS / FILL_WARPS;
constexpr int FILL_SLOTS = 128;
// SUPER: the Verlet-skin superset instead of the rows: a 5 x 5 x 5 cell
// stencil, every candidate within the pair radius plus the skin (FP32 with a
// margin: extra entries are removed by the exact filter later), up to SUP_W
// entries per particle in canonical order, and the positions they refer to.
// A row that does not fit marks the superset invalid, and this search's rows
// come from the exact form instead.
template <bool SUPER>
__global__ void __launch_bounds__(FILL_WARPS * 32) k_nbr_fill(DevPtrs P, DomainConst K) {
  if (SUPER) {
    if (!searching_full(P) || !K.skin_on) return;
  } else {
    if (!searching_full(P) || (K.skin_on && P.st->sup_valid && K.nspec == 0)) return;
  }
  // With the superset valid the filter forms the rows of the specimens that
  // search; this pass then only puts back the rows of those that do not.
  const bool keep_only = !SUPER && K.skin_on && P.st->sup_valid;
  __shared__ __align__(16) unsigned s_key[FILL_ROWS][FILL_SLOTS];
  __shared__ int s_idx[FILL_ROWS][FILL_SLOTS];
  __shared__ int s_len[FILL_ROWS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  size_t N = K.N;
  const int* ID = P.i + I_ID * N;
  const int* orig = P.i + I_ORIG * N;
  const int* kind = P.i + I_KIND * N;
  const int* material = P.i + I_MATERIAL * N;
  const int* cls = P.i + I_CLASS * N;
  const int ngroups = (K.N + FILL_ROWS - 1) / FILL_ROWS;
  unsigned long long pairs = 0;  // this warp's entries (lane 0), one atomic at the end
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
  const int i0 = grp * FILL_ROWS;
  // Each warp builds FILL_PER_WARP consecutive rows, one after the other, so
  // the block barrier below averages the warps' row costs over several rows.
  for (int rr = 0; rr < FILL_PER_WARP; ++rr) {
  const int row = w * FILL_PER_WARP + rr;
  const int i = i0 + row;
  unsigned* rkey = &s_key[row][0];
  int* ridx = &s_idx[row][0];
  int cnt = 0, split = 0;
  bool overflow = false, link = false;
  // A particle in a shadow bucket (non-finite position) has an empty row.
  const int key_i = i < K.N ? P.i[I_CELL * N + P.perm[i]] : 0;
  // Batched domain: a specimen that does not search keeps its rows (saved by
  // k_rows_save in canonical order; their keys here keep that order).
  const bool keep = !SUPER && K.nspec > 0 && i < K.N && !P.sp[P.i[I_SPEC * N + i]].do_search;
  if (keep_only && !keep) {
    if (lane == 0) s_len[row] = 0;
    continue;
  }
  if (keep) {
    const int old = P.perm[i];
    cnt = P.save_len[old];
    for (int e = lane; e < cnt; e += 32) {
      int v = P.save_nbr[(size_t)e * N + old];
      rkey[e] = (unsigned)e;
      ridx[e] = P.inv[v & 0x7fffffff] | (int)((unsigned)v & NB_UP);
    }
    __syncwarp();
  } else if (i < K.N && kind[i] == 0 && key_i < K.ncells) {
    float4 pi = reinterpret_cast<const float4*>(P.xs)[i];
    // The particle's cell: the key it was sorted by (k_cell_keys evaluated the
    // reference's FP64 cell formula once per particle), mapped back to grid
    // coordinates.
    int lin = P.cell_lin[key_i];
    int c[3] = {lin / (K.CellNo[1] * K.CellNo[2]), (lin / K.CellNo[2]) % K.CellNo[1], lin % K.CellNo[2]};
    int idi = ID[i], oi = orig[i], mi = material[i];
    bool ci = K.contact && is_contact_id(K, idi);
    const int spec_i = !SUPER && K.nspec > 0 ? P.i[I_SPEC * N + i] : 0;
    // Lane c < 27 fetches the range of neighbour cell c; a warp scan of the
    // counts flattens the candidates so all lanes work on every iteration.
    // A cell whose box lies farther from x_i than the largest pair radius
    // Cellfac * hmax holds no neighbour and is left out (about a quarter of
    // the candidates: most corner and some edge cells).  Boxes of the
    // outermost cells extend to infinity outwards, since the cell index is
    // clamped there.
    // The superset's stencil is 5 x 5 x 5 cells, taken 32 cells per round.
    constexpr int W = SUPER ? 5 : 3, NC = W * W * W, ROUNDS = (NC + 31) / 32;
    const float skip_r2 = SUPER ? K.sup_skip_r2 : K.cell_skip_r2;
    for (int round = 0; round < ROUNDS; ++round) {
    const int nq = NC - 32 * round < 32 ? NC - 32 * round : 32;  // stencil cells in this round
    const int qc = 32 * round + lane;
    int cs = 0, cc = 0;
    if (lane < nq) {
      int q3[3] = {c[0] + qc / (W * W) - W / 2, c[1] + (qc / W) % W - W / 2, c[2] + qc % W - W / 2};
      if (q3[0] >= 0 && q3[0] < K.CellNo[0] && q3[1] >= 0 && q3[1] < K.CellNo[1] && q3[2] >= 0 && q3[2] < K.CellNo[2]) {
        // FP32 on the prefilter coordinates x - BLPF (GB300 runs FP64 at 1/64
        // of the FP32 rate); the radius carries a margin above the FP32
        // rounding of those coordinates and of the cell bounds.
        const float xf[3] = {pi.x, pi.y, pi.z};
        float g2 = 0.f;
        bool inside = true;  // a particle outside the grid (clamped cell) keeps all 27 cells
        for (int d = 0; d < 3; ++d) {
          float lo = (float)q3[d] * K.CellSizef[d], hi = lo + K.CellSizef[d];
          float g = 0.f;
          if (q3[d] > 0 && xf[d] < lo) g = lo - xf[d];
          if (q3[d] < K.CellNo[d] - 1 && xf[d] > hi) g = xf[d] - hi;
          g2 += g * g;
          inside = inside && xf[d] >= 0.f && xf[d] <= (float)K.CellNo[d] * K.CellSizef[d];
        }
        if (!inside) g2 = 0.f;
        if (g2 <= skip_r2) {
          int key = P.cell_rank[(q3[0] * K.CellNo[1] + q3[1]) * K.CellNo[2] + q3[2]];
          cs = P.cell_start[key];
          cc = P.cell_start[key + 1] - cs;
        }
      }
    }
    int incl = cc;
    for (int off = 1; off < 32; off <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += v;
    }
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int excl = incl - cc;
    for (int base = 0; base < total; base += 32) {
      int t = base + lane;
      // cell of flat candidate t: the last lane q < 27 whose exclusive prefix
      // is <= t (prefixes are non-decreasing in q: binary search, 5 shuffles)
      int cell = 0;
      for (int step = 16; step > 0; step >>= 1) {
        int q = cell + step;
        int ex = __shfl_sync(0xffffffffu, excl, q < nq ? q : nq - 1);
        if (q < nq && ex <= t) cell = q;
      }
      int cstart = __shfl_sync(0xffffffffu, cs, cell);
      int cexcl = __shfl_sync(0xffffffffu, excl, cell);
      bool ok = false;
      unsigned kk = 0;
      int j = -1;
      if (t < total) {
        j = cstart + (t - cexcl);
        if (j != i) {
          int cj = cls[j];
          ok = !(K.contact && (ci || (cj & 2))) && (cj & 1) == 0 && (cj >> 2) == mi;
          if (ok) {
            float4 pj = reinterpret_cast<const float4*>(P.xs)[j];
            if (SUPER) {
              float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
              float Rs = K.half_cellfac_f * (pi.w + pj.w) + (float)K.skin;
              ok = dx * dx + dy * dy + dz * dz <= Rs * Rs * (1.0f + 4.0f * K.pre_eps);
            } else {
              ok = radius_ok(P, K, N, i, j, pi.x, pi.y, pi.z, pi.w, pj);
              if (ok && K.nspec > 0 && P.i[I_SPEC * N + j] != spec_i) link = true;
            }
          }
          if (ok) kk = (unsigned)(orig[j] - oi - 1);
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, ok);
      if (ok) {
        int pos = cnt + __popc(m & ((1u << lane) - 1u));
        // stored entry: the index, with bit 31 set when j has the larger
        // original index (P2 of the reference's (min, max) pair)
        if (pos < FILL_SLOTS) { rkey[pos] = kk; ridx[pos] = (int)((unsigned)j | (orig[j] > oi ? NB_UP : 0u)); }
      }
      cnt += __popc(m);
    }
    }  // stencil rounds
    if (cnt > (SUPER ? SUP_W : MAX_NB)) overflow = true;
    if (cnt > FILL_SLOTS) cnt = FILL_SLOTS;
    if (__any_sync(0xffffffffu, link) && lane == 0) atomicOr(&P.st->errors, ERR_SPEC_LINK);
  }
  // Order the row's slots by key.  Keys are distinct (one per neighbour), so
  // each entry's final slot is the number of smaller keys: every lane ranks
  // its own (at most four) entries against the whole row, read four keys per
  // broadcast load, then scatters them.  Pads above the row hold the largest
  // key, which no real key reaches (orig[j] - oi - 1 != -1).
  int cnt4 = (cnt + 3) & ~3;
  for (int e = cnt + lane; e < cnt4; e += 32) rkey[e] = 0xffffffffu;
  __syncwarp();
  const int nk = (cnt + 31) >> 5;  // warp-uniform
  unsigned key[4];
  int idx[4], rank[4] = {0, 0, 0, 0};
  for (int r = 0; r < 4; ++r) {
    int e = lane + 32 * r;
    key[r] = e < cnt ? rkey[e] : 0xffffffffu;
    idx[r] = e < cnt ? ridx[e] : 0;
  }
  if (nk <= 2) rank_row<2>(rkey, cnt4, key, rank);
  else rank_row<4>(rkey, cnt4, key, rank);
  __syncwarp();
  for (int r = 0; r < 4; ++r)
    if (lane + 32 * r < cnt) ridx[rank[r]] = idx[r];
  __syncwarp();
  if (SUPER) {
    if (i < K.N && lane == 0) {
      s_len[row] = cnt;
      P.sup_len[i] = cnt;
      if (overflow) P.st->sup_valid = 0;
      for (int d = 0; d < 3; ++d) P.xref[(size_t)d * N + i] = P.f[(C_X + d) * N + i];
    } else if (lane == 0) {
      s_len[row] = 0;
    }
    continue;
  }
  if (cnt > MAX_NB) cnt = MAX_NB;
  if (i < K.N) {
    for (int e = lane; e < cnt; e += 32) split += ridx[e] < 0 ? 1 : 0;
    for (int off = 16; off > 0; off >>= 1) split += __shfl_down_sync(0xffffffffu, split, off);
    if (lane == 0) {
      s_len[row] = cnt;
      P.row_len[i] = cnt;
      P.row_split[i] = split;
      P.i[I_NB * N + i] = cnt;
      if (K.contact) P.i[I_NWS * N + i] = (P.i[I_NWS * N + i] & 1) | ((ID[i] == K.id_free_surf) ? 2 : 0);
      if (overflow) atomicOr(&P.st->errors, ERR_NBR_OVERFLOW);
      if (!keep_only) pairs += (unsigned long long)cnt;  // the filter counts the kept rows
    }
  } else if (lane == 0) {
    s_len[row] = 0;
  }
  }  // rows of this warp
  __syncthreads();
  // Block-wide coalesced ELL write: thread (k, t) stores entry k of particle i0 + t.
  int maxlen = 0;
  for (int t = 0; t < FILL_ROWS; ++t) maxlen = max(maxlen, s_len[t]);
  if (SUPER) {  // superset rows are row-major (SUP_W entries per particle): a warp reads 32 in one line
    for (int q = threadIdx.x; q < FILL_ROWS * SUP_W; q += blockDim.x) {
      int t = q / SUP_W, k = q - t * SUP_W;
      if (k < s_len[t]) P.sup[(size_t)(i0 + t) * SUP_W + k] = s_idx[t][k];
    }
  } else {
    for (int q = threadIdx.x; q < maxlen * FILL_ROWS; q += blockDim.x) {
      int k = q / FILL_ROWS, t = q - k * FILL_ROWS;
      if (k < s_len[t]) P.nbr[(size_t)k * N + i0 + t] = s_idx[t][k];
    }
  }
  __syncthreads();  // the shared buffers are reused by the next group
  }
  if (!SUPER && lane == 0 && pairs) atomicAdd(&P.st->pair_count, pairs);
}

// ---- Verlet-skin reuse -------------------------------------------------------
// Largest squared displacement since the superset was built (a non-finite
// position gives NaN, whose bit pattern exceeds every finite one: a full
// search follows).
__global__ void k_skin_check(DevPtrs P, DomainConst K) {
  if (!searching(P) || !K.skin_on || !P.st->sup_valid) return;
  const size_t N = K.N;
  double m = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
    double d0 = P.f[(C_X + 0) * N + p] - P.xref[p];
    double d1 = P.f[(C_X + 1) * N + p] - P.xref[N + p];
    double d2 = P.f[(C_X + 2) * N + p] - P.xref[2 * N + p];
    double d = d0 * d0 + d1 * d1 + d2 * d2;
    if (!(d <= m)) m = d;
  }
  unsigned long long b = (unsigned long long)__double_as_longlong(m);
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
    b = o > b ? o : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(&P.st->maxdisp2_bits, b);
}

// Full search or filter only: a filter suffices while every particle has
// moved less than skin / 2 since the superset was built, since a pair within
// its radius now was then within the radius plus the skin.
__global__ void k_search_mode(DevPtrs P, DomainConst K) {
  StepState* s = P.st;
  if (!s->do_search) return;
  const double md2 = __longlong_as_double((long long)s->maxdisp2_bits);
  const double half = 0.5 * K.skin;
  const bool filter_only = K.skin_on && s->sup_valid && md2 <= half * half;
  s->search_full = filter_only ? 0 : 1;
  if (!filter_only) {
    s->nb_full_searches += 1;
    if (K.skin_on) s->sup_valid = 1;  // the superset build clears it again if a row does not fit
  }
}

// Cell coordinates at the current positions (ListGenerate's clamped cell
// index, Neighbour.cpp:185-218, the same FP64 expression as k_cell_keys),
// 21 bits per axis, -1 for a non-finite position; and the FP32 prefilter
// coordinates.  COVER: the filter leaves the cell test out, so only the
// finiteness is recorded.  In a batched domain only the particles of the
// specimens that search are needed (no pair leaves a specimen).
template <bool COVER>
__global__ void k_cell_coords(DevPtrs P, DomainConst K) {
  if (!searching(P) || !K.skin_on || !P.st->sup_valid) return;
  const size_t N = K.N;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.N; p += gridDim.x * blockDim.x) {
    if (K.nspec > 0 && !P.sp[P.i[I_SPEC * N + p]].do_search) continue;
    long long code = 0;
    bool finite = true;
    for (int d = 0; d < 3; ++d) {
      double xd = P.f[(C_X + d) * N + p];
      finite = finite && isfinite(xd);
      if (!COVER) {
        int q = (int)floor(__ddiv_rn(__dsub_rn(xd, K.BLPF[d]), K.CellSize[d]));
        if (q < 0) q = 0;
        if (q >= K.CellNo[d]) q = K.CellNo[d] - 1;
        code = (code << 21) | (long long)q;
      }
    }
    P.cellc[p] = finite ? code : -1;
    reinterpret_cast<float4*>(P.xs)[p] =
        make_float4((float)(P.f[(C_X + 0) * N + p] - K.BLPF[0]), (float)(P.f[(C_X + 1) * N + p] - K.BLPF[1]),
                    (float)(P.f[(C_X + 2) * N + p] - K.BLPF[2]), (float)P.f[C_H * N + p]);
  }
}

__device__ __forceinline__ bool cells_adjacent(long long a, long long b) {
  for (int d = 0; d < 3; ++d) {
    int qa = (int)((a >> (21 * d)) & 0x1fffff), qb = (int)((b >> (21 * d)) & 0x1fffff);
    if (qa - qb > 1 || qb - qa > 1) return false;
  }
  return true;
}

// Rows from the superset: the entries whose particles sit in adjacent cells
// now and pass the radius rule (FP32 prefilter, exact FP64 CheckRadius),
// in the superset's canonical order — the rows a full search gives.
// COVER: every cell is wider than the largest pair radius (DomainConst::
// cells_cover), so a pair that passes the radius rule is in adjacent cells
// and the cell test is left out (a non-finite position fails the radius rule).
// One warp per particle, 32 superset entries per round (one coalesced line of
// the row-major superset); the kept entries are compacted by ballot in order
// into shared memory, and the block writes its FILL_ROWS rows to the ELL
// array one coalesced line per entry index.  In a batched domain the rows of
// specimens that do not search stay as they are (untouched, or put back by
// k_nbr_fill after a reordering).
template <bool COVER>
__global__ void __launch_bounds__(FILL_WARPS * 32, 4) k_nbr_filter(DevPtrs P, DomainConst K) {
  if (!searching(P) || !K.skin_on || !P.st->sup_valid) return;
  __shared__ int s_idx[FILL_ROWS][MAX_NB];
  __shared__ int s_len[FILL_ROWS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t N = K.N;
  const float4* xs = reinterpret_cast<const float4*>(P.xs);
  const int ngroups = (K.N + FILL_ROWS - 1) / FILL_ROWS;
  unsigned long long pairs = 0;  // this warp's entries (lane 0), one atomic at the end
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int i0 = grp * FILL_ROWS;
    for (int rr = 0; rr < FILL_PER_WARP; ++rr) {
      const int row = w * FILL_PER_WARP + rr;
      const int i = i0 + row;
      int cnt = 0;
      if (K.nspec > 0 && i < K.N && !P.sp[P.i[I_SPEC * N + i]].do_search) {
        if (lane == 0) { s_len[row] = 0; pairs += (unsigned long long)P.row_len[i]; }
        continue;
      }
      const int spec_i = K.nspec > 0 && i < K.N ? P.i[I_SPEC * N + i] : 0;
      bool link = false;
      const long long ci = i < K.N ? P.cellc[i] : -1;
      if (i < K.N && P.i[I_KIND * N + i] == 0 && ci >= 0) {
        const float4 pi = xs[i];
        const int len = P.sup_len[i];
        const int* sr = P.sup + (size_t)i * SUP_W;
        // All of the row's loads are issued before any is used: the lane's up
        // to four entries (k = lane + 32 r), then their positions, so a row
        // costs two memory latencies rather than two per 32 entries.
        constexpr int R = SUP_W / 32;
        int e[R];
        float4 pj[R];
        long long cj[R];
#pragma unroll
        for (int r = 0; r < R; ++r) e[r] = lane + 32 * r < len ? sr[lane + 32 * r] : 0;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (lane + 32 * r < len) {
            pj[r] = xs[nb_index(e[r])];
            if (!COVER) cj[r] = P.cellc[nb_index(e[r])];
          }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (32 * r >= len) break;  // warp-uniform
          bool ok = false;
          if (lane + 32 * r < len) {
            ok = COVER || (cj[r] >= 0 && cells_adjacent(ci, cj[r]));
            if (ok) ok = radius_ok(P, K, N, i, nb_index(e[r]), pi.x, pi.y, pi.z, pi.w, pj[r]);
            if (ok && K.nspec > 0 && P.i[I_SPEC * N + nb_index(e[r])] != spec_i) link = true;
          }
          const unsigned m = __ballot_sync(0xffffffffu, ok);
          if (ok) {
            const int pos = cnt + __popc(m & ((1u << lane) - 1u));
            if (pos < MAX_NB) s_idx[row][pos] = e[r];
          }
          cnt += __popc(m);
        }
      }
      if (cnt > MAX_NB && lane == 0) atomicOr(&P.st->errors, ERR_NBR_OVERFLOW);
      if (__any_sync(0xffffffffu, link) && lane == 0) atomicOr(&P.st->errors, ERR_SPEC_LINK);
      if (cnt > MAX_NB) cnt = MAX_NB;
      __syncwarp();
      int split = 0;
      for (int e = lane; e < cnt; e += 32) split += s_idx[row][e] < 0 ? 1 : 0;
      for (int off = 16; off > 0; off >>= 1) split += __shfl_down_sync(0xffffffffu, split, off);
      if (lane == 0) {
        s_len[row] = i < K.N ? cnt : 0;
        if (i < K.N) {
          P.row_len[i] = cnt;
          P.row_split[i] = split;
          P.i[I_NB * N + i] = cnt;
          pairs += (unsigned long long)cnt;
        }
      }
    }
    __syncthreads();
    int maxlen = 0;
    for (int t = 0; t < FILL_ROWS; ++t) maxlen = max(maxlen, s_len[t]);
    for (int q = threadIdx.x; q < maxlen * FILL_ROWS; q += blockDim.x) {
      int k = q / FILL_ROWS, t = q - k * FILL_ROWS;
      if (k < s_len[t]) P.nbr[(size_t)k * N + i0 + t] = s_idx[t][k];
    }
    __syncthreads();  // the shared rows are reused by the next group
  }
  if (lane == 0 && pairs) atomicAdd(&P.st->pair_count, pairs);
}

// CalculateSurface (Domain.cpp:1415-1491): n_i = sum_j m_j (x_i - x_j) in row
// order; |n| / totmass >= 0.25 h and Nb <= 46 marks the free surface (ID 1).
__global__ void k_surface(DevPtrs P, DomainConst K) {
  if (!searching(P)) return;
  size_t N = K.N;
  unsigned nsurf = 0;  // summed over the warp, one atomic per warp
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K.N; i += gridDim.x * blockDim.x) {
  if (P.i[I_KIND * N + i] != 0) continue;
  double xi = P.f[C_X * N + i], yi = P.f[(C_X + 1) * N + i], zi = P.f[(C_X + 2) * N + i];
  double n0 = 0, n1 = 0, n2 = 0;
  int len = P.row_len[i];
  for (int k = 0; k < len; ++k) {
    int j = nb_index(P.nbr[(size_t)k * N + i]);
    double mj = P.f[C_MASS * N + j];
    n0 = __dadd_rn(n0, __dmul_rn(mj, __dsub_rn(xi, P.f[C_X * N + j])));
    n1 = __dadd_rn(n1, __dmul_rn(mj, __dsub_rn(yi, P.f[(C_X + 1) * N + j])));
    n2 = __dadd_rn(n2, __dmul_rn(mj, __dsub_rn(zi, P.f[(C_X + 2) * N + j])));
  }
  double s = __ddiv_rn(1.0, K.totmass_mean);
  n0 = __dmul_rn(s, n0); n1 = __dmul_rn(s, n1); n2 = __dmul_rn(s, n2);
  P.f[C_NORMAL * N + i] = n0; P.f[(C_NORMAL + 1) * N + i] = n1; P.f[(C_NORMAL + 2) * N + i] = n2;
  int id = P.i[I_IDORIG * N + i];
  double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(n0, n0), __dmul_rn(n1, n1)), __dmul_rn(n2, n2)));
  bool surf = (nn >= __dmul_rn(0.25, P.f[C_H * N + i])) && (len <= 46);
  if (surf) {
    if (!(P.i[I_NWS * N + i] & 1)) id = 1;
    ++nsurf;
  }
  P.i[I_ID * N + i] = id;
  }
  nsurf = __reduce_add_sync(0xffffffffu, nsurf);
  if ((threadIdx.x & 31) == 0 && nsurf) atomicAdd(&P.st->surface_count, (int)nsurf);
}

// ContactNbSearch (Contact.cpp:57-132): surface particle (at search time and
// now) within h1 + h2 of a rigid-mesh particle in a neighbouring cell.
// Row sorted by the mesh particle's original index.
__global__ void k_contact_pairs(DevPtrs P, DomainConst K) {
  if (!searching(P)) return;
  size_t N = K.N;
  unsigned npairs = 0;  // summed over the warp, one atomic per warp
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K.N; i += gridDim.x * blockDim.x) {
  int cnt = 0;
  bool overflow = false;
  int row[MAX_CP];
  int keys[MAX_CP];
  int idi = P.i[I_ID * N + i];
  bool ok = P.i[I_KIND * N + i] == 0 && (P.i[I_NWS * N + i] & 2) && idi == K.id_free_surf;
  if (ok) {
    double xi = P.f[C_X * N + i], yi = P.f[(C_X + 1) * N + i], zi = P.f[(C_X + 2) * N + i];
    double hi = P.f[C_H * N + i];
    int c[3];
    for (int d = 0; d < 3; ++d) {
      int q = (int)floor(__ddiv_rn(__dsub_rn(P.f[(C_X + d) * N + i], K.BLPF[d]), K.CellSize[d]));
      c[d] = q < 0 ? 0 : (q >= K.CellNo[d] ? K.CellNo[d] - 1 : q);
    }
    for (int a = c[0] - 1; a <= c[0] + 1; ++a) {
      if (a < 0 || a >= K.CellNo[0]) continue;
      for (int b = c[1] - 1; b <= c[1] + 1; ++b) {
        if (b < 0 || b >= K.CellNo[1]) continue;
        for (int e = c[2] - 1; e <= c[2] + 1; ++e) {
          if (e < 0 || e >= K.CellNo[2]) continue;
          int key = P.cell_rank[(a * K.CellNo[1] + b) * K.CellNo[2] + e];
          for (int j = P.cell_start[key]; j < P.cell_start[key + 1]; ++j) {
            if (P.i[I_KIND * N + j] != 1) continue;
            if (!is_contact_id(K, P.i[I_ID * N + j])) continue;
            double dx = __dsub_rn(xi, P.f[C_X * N + j]), dy = __dsub_rn(yi, P.f[(C_X + 1) * N + j]),
                   dz = __dsub_rn(zi, P.f[(C_X + 2) * N + j]);
            double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
            if (!(r < __dadd_rn(hi, P.f[C_H * N + j]))) continue;
            int kk = P.i[I_ORIG * N + j];
            if (cnt < MAX_CP) {
              int m = cnt - 1;
              while (m >= 0 && keys[m] > kk) { keys[m + 1] = keys[m]; row[m + 1] = row[m]; --m; }
              keys[m + 1] = kk; row[m + 1] = j;
              ++cnt;
            } else overflow = true;
          }
        }
      }
    }
  }
  for (int k = 0; k < cnt; ++k) P.cp[(size_t)k * N + i] = row[k];
  P.cp_len[i] = cnt;
  if (overflow) atomicOr(&P.st->errors, ERR_CONTACT_OVERFLOW);
  npairs += (unsigned)cnt;
  }
  npairs = __reduce_add_sync(0xffffffffu, npairs);
  if ((threadIdx.x & 31) == 0 && npairs) atomicAdd(&P.st->contact_pair_count, (unsigned long long)npairs);
}

__global__ void k_force_search(DevPtrs P) { P.st->do_search = 1; }
void launch_force_search(const DevPtrs& P, cudaStream_t s) { k_force_search<<<1, 1, 0, s>>>(P); }

__global__ void k_search_begin(DevPtrs P) {
  if (!searching(P)) return;
  P.st->pair_count = 0;
  P.st->contact_pair_count = 0;
  P.st->surface_count = 0;
  P.st->nan_count = 0;
  P.st->maxdisp2_bits = 0;
  P.st->nb_searches += 1;
}

// ---------------------------------------------------------------- host side
static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

void launch_neighbour_search(const DevPtrs& P, const DomainConst& K, double* fscratch, int* iscratch,
                             cudaStream_t s) {
  const int T = 256;
  // Gated kernels run on fixed grids with grid-stride loops: on steps that do
  // not search, each launch is a handful of blocks that exit at once.
  const int G = 152 * 4;
  auto grid = [&](long long n) { int b = nblk(n, T); return b < G ? b : G; };
  // buckets: ncells grid cells (Morton ranks), then ncells shadow buckets
  const long long nbk = 2LL * K.ncells;
  int nz = grid(nbk);
  k_search_begin<<<1, 1, 0, s>>>(P);
  mark(s, "k_search_begin");
  if (K.skin_on) {
    k_skin_check<<<grid(K.N), T, 0, s>>>(P, K);
    mark(s, "k_skin_check");
  }
  k_search_mode<<<1, 1, 0, s>>>(P, K);
  mark(s, "k_search_mode");
  if (K.nspec > 0) {
    k_rows_save<<<grid(K.N), T, 0, s>>>(P, K);
    mark(s, "k_rows_save");
  }
  k_zero_int<<<nz, T, 0, s>>>(P, P.cell_count, nbk, 1);
  mark(s, "k_zero_int");
  k_cell_keys<<<grid(K.N), T, 0, s>>>(P, K);
  mark(s, "k_cell_keys");
  int nb = nblk(nbk, SCAN_TILE);
  k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(P, P.cell_count, nbk, P.scan_tmp);
  mark(s, "k_scan_reduce");
  k_scan_top<<<1, SCAN_THREADS, 0, s>>>(P, P.scan_tmp, nb);
  mark(s, "k_scan_top");
  k_scan_down<<<nb, SCAN_THREADS, 0, s>>>(P, P.cell_count, nbk, P.scan_tmp, P.cell_start, P.cell_start + nbk);
  mark(s, "k_scan_down");
  k_zero_int<<<nz, T, 0, s>>>(P, P.cell_count, nbk, 1);
  mark(s, "k_zero_int");
  k_scatter<<<grid(K.N), T, 0, s>>>(P, K);
  mark(s, "k_scatter");
  k_sort_cells<<<grid(nbk), T, 0, s>>>(P, K);
  mark(s, "k_sort_cells");
  k_permute<<<152 * 4, 512, 0, s>>>(P, K, fscratch, iscratch);
  mark(s, "k_permute");
  k_copy_back<<<152 * 4, 512, 0, s>>>(P, K, fscratch, iscratch);
  mark(s, "k_copy_back");
  k_after_permute<<<grid(K.N), T, 0, s>>>(P, K);
  mark(s, "k_after_permute");
  {
    // a few resident blocks per SM, striding over the row groups
    int groups = nblk(K.N, FILL_ROWS), cap = 152 * 4;
    if (K.skin_on) {
      k_nbr_fill<true><<<groups < cap ? groups : cap, FILL_WARPS * 32, 0, s>>>(P, K);
      mark(s, "k_sup_build");
    }
    k_nbr_fill<false><<<groups < cap ? groups : cap, FILL_WARPS * 32, 0, s>>>(P, K);
  }
  mark(s, "k_nbr_fill");
  if (K.skin_on) {
    if (K.cells_cover) k_cell_coords<true><<<grid(K.N), T, 0, s>>>(P, K);
    else k_cell_coords<false><<<grid(K.N), T, 0, s>>>(P, K);
    mark(s, "k_cell_coords");
    int groups = nblk(K.N, FILL_ROWS), cap = 152 * 4;
    if (K.cells_cover) k_nbr_filter<true><<<groups < cap ? groups : cap, FILL_WARPS * 32, 0, s>>>(P, K);
    else k_nbr_filter<false><<<groups < cap ? groups : cap, FILL_WARPS * 32, 0, s>>>(P, K);
    mark(s, "k_nbr_filter");
  }
  if (P.halo) launch_halo_build(P, K, s);
  if (K.contact) {
    k_surface<<<grid(K.N), T, 0, s>>>(P, K);
    mark(s, "k_surface");
    k_contact_pairs<<<grid(K.N), 128, 0, s>>>(P, K);
    mark(s, "k_contact_pairs");
  }
}

}  // namespace wf
