// Neighbour-list and pair-list rebuilds (replace update_neighbor_list /
// update_pair_list, sop.cu:704-920, 928-1262, 1456-1706, and the CUDPP radix
// sort + scan they use).
//
// Neighbour list (every nnlup steps):
//   1. per-molecule bounding box of the coordinates             k_bbox
//   2. per-molecule cell grid (cell edge rc/S, S=1..3 chosen so a cell holds
//      ~4 beads; S=1..4 and ~1 bead from 10,000 beads up; molecules whose
//      extent + rc reaches boxl, where the minimum image matters, fall back
//      to index-chunked cells that scan all pairs)
//                                                                k_grid, k_grid_base
//   3. counting sort of beads into cells (own scan), cells sorted by bead id
//      so every later order is deterministic, coordinates staged in that
//      order                             k_assign, scan, k_scatter, k_cellsort, k_stage_xs
//   4. 8 lanes per bead in cell order: the bead against the beads of the
//      cell rows within S along each axis, culled to its own cut-off sphere;
//      predicate = the reference's FP32 host filter (d^2 < rcut^2, |i-j| > 2,
//      not native); one pass writes fixed-stride rows (overflow: regrow) k_nl
//   The attractive neighbour list filters each bead's native row (k_assign).
// Pair list (every nplup steps): eight lanes per bead, beads in chain order,
// compact its neighbour-list row in row order (k_pl).
#include "sop_dev.cuh"

namespace sop {

// ------------------------------------------------------------------ scan
// Exclusive scan of n ints: out[0..n], out[n] = total.  Three kernels:
// per-block reduce, one-block scan of the block sums, per-block apply.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and the block total in *total.  The total has its own slot: with
// 1,024 threads all 32 warp slots hold prefixes.
__device__ __forceinline__ int block_excl_scan(int v, int* total) {
  __shared__ int warp_sums[32];
  __shared__ int block_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = warp_incl_scan(v);
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    int s = lane < nw ? warp_sums[lane] : 0;
    int si = warp_incl_scan(s);
    if (lane < nw) warp_sums[lane] = si - s;
    if (lane == 31) block_total = si;
  }
  __syncthreads();
  int res = incl - v + warp_sums[w];
  *total = block_total;
  __syncthreads();
  return res;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int* __restrict__ in, long long n,
                                                               int* __restrict__ block_sums) {
  long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += in[base + k];
  int total;
  block_excl_scan(s, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_top(int* __restrict__ block_sums, int nblocks) {
  int carry = 0;
  for (int b0 = 0; b0 < nblocks; b0 += blockDim.x) {
    int b = b0 + threadIdx.x;
    int v = b < nblocks ? block_sums[b] : 0;
    int total;
    int ex = block_excl_scan(v, &total);
    if (b < nblocks) block_sums[b] = ex + carry;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ in, long long n,
                                                              const int* __restrict__ block_sums,
                                                              int* __restrict__ out) {
  long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int ex = block_excl_scan(s, &total) + block_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = ex;
    ex += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = ex;
}

// ---------------------------------------------------------------- grids
// Each binning kernel's work per item is a device function, so that the
// kernels below and the one-block binning of small contexts (k_bin_small)
// share it.
__device__ __forceinline__ void bbox_reset_at(const DevSys& s, int m) {
  if (m >= s.nmol) return;
  unsigned* b = s.bbox + 6 * m;
  b[0] = b[1] = b[2] = f2ord(INFINITY);
  b[3] = b[4] = b[5] = f2ord(-INFINITY);
}
__global__ void k_bbox_reset(DevSys s) { bbox_reset_at(s, blockIdx.x * blockDim.x + threadIdx.x); }

// Molecules whose lists a rebuild at block offset koff refreshes: running,
// healthy, and with the step this rebuild precedes (mol_step + koff + 1)
// still within the step budget -- a molecule that has finished keeps the
// lists of its last step, as the reference's loop ends there.
__device__ __forceinline__ bool mol_listed(const DevSys& s, int m, int koff) {
  if (m < 0) return false;
  if (s.only_mol >= 0 && m != s.only_mol) return false;  // its lists and grid stay
  const MolConst& mc = s.mol[m];
  return mc.active && s.mol_status[m] == 0 &&
         !(mc.nsteps >= 0 && s.mol_step[m] + koff >= mc.nsteps);
}

// Coordinates at step mol_step + koff (the positions the rebuild uses).
__device__ __forceinline__ const float4* xbuf(const DevSys& s, int m, int koff) {
  return s.x[(int)((s.mol_step[m] + koff) & 1)];
}

// Called by all 32 lanes of a warp together (warp votes).
__device__ __forceinline__ void bbox_at(const DevSys& s, int koff, int i) {
  int m = (i < s.nlive) ? s.mol_of[i] : -1;
  bool ok = mol_listed(s, m, koff);
  unsigned act = __ballot_sync(0xffffffffu, ok);
  if (!ok) return;
  float4 x = xbuf(s, m, koff)[i];
  unsigned peers = __match_any_sync(act, m);
  unsigned lo[3] = {f2ord(x.x), f2ord(x.y), f2ord(x.z)};
  unsigned mn[3], mx[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    mn[a] = __reduce_min_sync(peers, lo[a]);
    mx[a] = __reduce_max_sync(peers, lo[a]);
  }
  if ((threadIdx.x & 31) == __ffs(peers) - 1) {
    unsigned* b = s.bbox + 6 * m;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(b + a, mn[a]);
      atomicMax(b + 3 + a, mx[a]);
    }
  }
}
__global__ void k_bbox(DevSys s, int koff) { bbox_at(s, koff, blockIdx.x * blockDim.x + threadIdx.x); }

// One thread per molecule: cell grid of its neighbour-list build.
__device__ __forceinline__ void grid_at(const DevSys& s, int* ncell, int koff, int m) {
  if (m >= s.nmol) return;
  if (s.only_mol >= 0 && m != s.only_mol) {  // a rebuild of another molecule alone
    ncell[m] = 0;
    return;
  }
  MolGrid g = {};
  int n = s.mol[m].n;
  if (!mol_listed(s, m, koff) || n <= 0) {
    g.ncell = 0;
    s.grid[m] = g;
    ncell[m] = 0;
    return;
  }
  // the bounds come from atomics (performed in L2): read them from L2, so
  // that a block that reset them itself cannot see its own stale L1 lines
  const unsigned* b = s.bbox + 6 * m;
  float lo[3], ext[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = ord2f(__ldcg(b + a));
    ext[a] = ord2f(__ldcg(b + 3 + a)) - lo[a];
  }
  const float rc = s.rc_nl_rep_max;
  bool periodic = false;
  for (int a = 0; a < 3; ++a) periodic |= !(ext[a] + rc < s.boxl);  // also true for NaN extents
  // Separations inside the box [lo, lo + ext] never exceed ext (rounding is
  // monotone), so below boxl/4 the minimum image leaves them unchanged.  The
  // margin of one cut-off covers the drift until the next rebuild, for the
  // pair-list filters that use the same flag.
  bool wrap = false;
  for (int a = 0; a < 3; ++a) wrap |= !(ext[a] + rc < 0.25f * s.boxl);
  if (periodic || n <= 96) {
    // every pair is scanned; cells are chunks of 32 consecutive beads
    g.brute = 1;
    g.dims[0] = (n + 31) / 32; g.dims[1] = 1; g.dims[2] = 1;
    g.S = g.dims[0];
    g.cs = 0.0f;
    g.lo[0] = g.lo[1] = g.lo[2] = 0.0f;
  } else {
    float vol = fmaxf((ext[0] + 1.0f) * (ext[1] + 1.0f) * (ext[2] + 1.0f), 1.0f);
    float rho = (float)n / vol;
    // about 4 beads per cell (S <= 3); a molecule of 10,000 beads or more
    // scans enough cells per bead that finer ones (about 1 bead, S <= 4) cull
    // more candidates than they add rows
    const bool big = n >= 10000;
    const int smax = big ? 4 : 3;
    int S = (int)floorf(rc * cbrtf(rho * (big ? 1.0f : 0.25f)));
    S = S < 1 ? 1 : (S > smax ? smax : S);
    float cs = rc * 1.0001f / (float)S + 1.0e-4f;
    long long cap = n * 2 > 64 ? (long long)n * 2 : 64;
    for (int iter = 0; iter < 8; ++iter) {
      long long tot = 1;
      for (int a = 0; a < 3; ++a) {
        g.dims[a] = (int)floorf(ext[a] / cs) + 1;
        tot *= g.dims[a];
      }
      if (tot <= cap) break;
      cs *= cbrtf((float)tot / (float)cap) * 1.01f;
      S = (int)ceilf(rc * 1.0001f / cs);
      if (S < 1) S = 1;
    }
    g.brute = 0;
    g.S = S;
    g.cs = cs;
    for (int a = 0; a < 3; ++a) g.lo[a] = lo[a];
  }
  g.wrap = wrap ? 1 : 0;
  g.ncell = g.dims[0] * g.dims[1] * g.dims[2];
  s.grid[m] = g;
  ncell[m] = g.ncell;
}
__global__ void k_grid(DevSys s, int* __restrict__ ncell, int koff) {
  grid_at(s, ncell, koff, blockIdx.x * blockDim.x + threadIdx.x);
}

// Single block: cell bases = exclusive scan of the per-molecule cell counts;
// flags overflow of the cell capacity (cannot happen by construction: each
// molecule holds at most max(64, 2n) cells, and the capacity is their sum).
// Called by every thread of one block.
__device__ __forceinline__ void grid_base_block(const DevSys& s, const int* ncell, int* cells_total) {
  int carry = 0;
  for (int b0 = 0; b0 < s.nmol; b0 += blockDim.x) {
    int m = b0 + threadIdx.x;
    int v = m < s.nmol ? ncell[m] : 0;
    int total;
    int ex = block_excl_scan(v, &total);
    if (m < s.nmol) s.grid[m].base = ex + carry;
    carry += total;
  }
  if (threadIdx.x == 0) {
    if (carry > s.cell_cap) atomicOr(s.flags, FLAG_NL_OVERFLOW);
    *cells_total = carry > s.cell_cap ? (int)s.cell_cap : carry;
  }
}
__global__ void __launch_bounds__(1024) k_grid_base(DevSys s, const int* __restrict__ ncell,
                                                     int* __restrict__ cells_total) {
  grid_base_block(s, ncell, cells_total);
}

__device__ __forceinline__ int cell_coord(float v, float lo, float cs, int dim) {
  int c = (int)floorf((v - lo) / cs);
  return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

// Per bead: cell index and slot (counting sort), plus the attractive
// neighbour-list filter of its native row (sop.cu:704-759 semantics).
__device__ __forceinline__ void assign_at(const DevSys& s, int koff, int att, int i) {
  if (i >= s.nlive) return;
  int m = s.mol_of[i];
  if (!mol_listed(s, m, koff)) {  // not binned; its lists stay as they are
    s.bead_cell[i] = -1;
    return;
  }
  const float4* X = xbuf(s, m, koff);
  float4 xi = X[i];
  MolGrid g = s.grid[m];
  int c;
  if (g.brute) {
    c = g.base + (i - s.mol[m].start) / 32;
  } else {
    int cx = cell_coord(xi.x, g.lo[0], g.cs, g.dims[0]);
    int cy = cell_coord(xi.y, g.lo[1], g.cs, g.dims[1]);
    int cz = cell_coord(xi.z, g.lo[2], g.cs, g.dims[2]);
    c = g.base + (cz * g.dims[1] + cy) * g.dims[0] + cx;
  }
  if (c < 0 || c >= s.cell_cap) {  // unreachable: capacity is the sum of the per-molecule caps
    atomicOr(s.flags, FLAG_NL_OVERFLOW);
    s.bead_cell[i] = -1;
    s.nl_att_cnt[i] = 0;
    return;
  }
  s.bead_cell[i] = c;
  s.bead_slot[i] = atomicAdd(s.cell_cnt + c, 1);
  if (!att) return;  // binning only: the lists stay as they are
  int2 row = s.nat_row[i];
  int k = 0;
  for (int e = 0; e < row.y; ++e) {
    int idx = row.x + e;
    float4 xj = X[s.nat_j[idx]];
    float dx = __fsub_rn(xj.x, xi.x), dy = __fsub_rn(xj.y, xi.y),
          dz = __fsub_rn(xj.z, xi.z);
    min_image3(dx, dy, dz, s.boxl);
    if (d2_exact(dx, dy, dz) < s.nat_rc2[idx].x) s.nl_att_e[row.x + k++] = idx;
  }
  s.nl_att_cnt[i] = k;
}
__global__ void k_assign(DevSys s, int koff, int att) {
  assign_at(s, koff, att, blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ void scatter_at(const DevSys& s, int i) {
  if (i >= s.nlive) return;
  int c = s.bead_cell[i];
  if (c < 0) return;
  s.sorted[s.cell_start[c] + s.bead_slot[i]] = i;
}
__global__ void k_scatter(DevSys s) { scatter_at(s, blockIdx.x * blockDim.x + threadIdx.x); }

// Per cell: sort its beads by id (fixes every downstream order).  Cells hold
// a handful of beads, so one thread's insertion sort is short.
__device__ __forceinline__ void cellsort_at(const DevSys& s, const int* cells_total, long long c) {
  if (c >= *cells_total) return;
  int cnt = __ldcg(s.cell_cnt + c);  // counted by atomics: read from L2
  if (cnt == 0) return;
  int* b = s.sorted + s.cell_start[c];
  for (int a = 1; a < cnt; ++a) {
    int v = b[a], k = a;
    while (k > 0 && b[k - 1] > v) { b[k] = b[k - 1]; --k; }
    b[k] = v;
  }
}
__global__ void k_cellsort(DevSys s, const int* __restrict__ cells_total) {
  cellsort_at(s, cells_total, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Coordinates staged in cell order, w = (id << 2) | type: a thread per
// position, so the gathers are independent.
__device__ __forceinline__ void stage_xs_at(const DevSys& s, int koff, int k) {
  if (k >= s.cell_start[s.cell_cap]) return;  // beads that were binned
  const int i = s.sorted[k];
  float4 x = xbuf(s, s.mol_of[i], koff)[i];
  x.w = __int_as_float((i << 2) | type_of(x));
  s.xs[k] = x;
}
__global__ void k_stage_xs(DevSys s, int koff) { stage_xs_at(s, koff, blockIdx.x * blockDim.x + threadIdx.x); }

// The whole binning in one block, for contexts small enough that the chain of
// kernels above costs mostly launch latency: the same per-item work, phase
// by phase, with block barriers between phases, so the same cells, order
// and coordinates.  The scan of the cell counts runs over the block.
constexpr int kBinThreads = 1024;
constexpr long long kBinSmallCells = 1 << 16;
//
// Values that atomics produced in this kernel (the molecule bounds, the cell
// counts) are read with __ldcg: atomics complete in L2, and the block's own
// L1 may still hold the lines it cleared before them.
__global__ void __launch_bounds__(kBinThreads) k_bin_small(DevSys s, int* ncell, int* cells_total,
                                                           int koff, int att) {
  const int t = threadIdx.x;
  for (int m = t; m < s.nmol; m += kBinThreads) bbox_reset_at(s, m);
  __syncthreads();
  // every lane of a warp takes part in each round (warp votes)
  for (int i0 = 0; i0 < s.nlive; i0 += kBinThreads) bbox_at(s, koff, i0 + t);
  __syncthreads();
  for (int m = t; m < s.nmol; m += kBinThreads) grid_at(s, ncell, koff, m);
  __syncthreads();
  grid_base_block(s, ncell, cells_total);
  for (long long c = t; c < s.cell_cap; c += kBinThreads) s.cell_cnt[c] = 0;
  __syncthreads();
  for (int i = t; i < s.nlive; i += kBinThreads) assign_at(s, koff, att, i);
  __syncthreads();
  int carry = 0;  // exclusive scan of the cell counts into cell_start
  for (long long c0 = 0; c0 < s.cell_cap; c0 += kBinThreads) {
    const long long c = c0 + t;
    const int v = c < s.cell_cap ? __ldcg(s.cell_cnt + c) : 0;
    int total;
    const int ex = block_excl_scan(v, &total);
    if (c < s.cell_cap) s.cell_start[c] = carry + ex;
    carry += total;
  }
  if (t == 0) s.cell_start[s.cell_cap] = carry;
  __syncthreads();
  for (int i = t; i < s.nlive; i += kBinThreads) scatter_at(s, i);
  __syncthreads();
  for (long long c = t; c < s.cell_cap; c += kBinThreads) cellsort_at(s, cells_total, c);
  __syncthreads();
  for (int k = t; k < s.nlive; k += kBinThreads) stage_xs_at(s, koff, k);
}

// The lanes of a group of L lanes (L divides 32) within its warp.
template <int L>
__device__ __forceinline__ unsigned group_mask(int wl) {
  return L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (wl & ~(L - 1)));
}

// Contexts of up to this many bead slots rebuild their lists with a warp
// per bead: at 8 lanes per bead they fill less than a wave of the GPU.
constexpr int kWideListBeads = 16384;

constexpr int kNatRegs = 16;  // native partners held in registers (the rest are read)

// Distance from v to the slab [a, a + w] (0 inside).
// cell_coord with a multiply by the inverse edge: for bounds that carry a
// margin far above its rounding (about 1e-5 cells)
__device__ __forceinline__ int cell_coord_fast(float v, float lo, float inv_cs, int dim) {
  int c = (int)floorf((v - lo) * inv_cs);
  return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

__device__ __forceinline__ float slab_dist(float v, float a, float w) {
  return fmaxf(fmaxf(a - v, v - (a + w)), 0.0f);
}

// L lanes per bead (8, or a warp for small contexts; the rows do not depend
// on L), beads in cell order (xs), so neighbouring groups
// share cells and candidates.  Each bead scans the cell rows (runs along x)
// of its grid neighbourhood, culled against its own position: rows whose
// y,z slab lies beyond the cut-off are skipped and each row's x range is
// clipped to the chord.  Partners that pass the reference's predicate
// (sop.cu:768-826 with the host arithmetic of sop.cu:1414-1435:
// d^2 < (fac*sigma or abs)^2 in FP32, |i - j| > 2, not a native contact) are
// written to the bead's fixed-stride row in candidate order (group ballot).
// The culling is conservative (a 1e-3 A margin); membership is decided by the
// exact predicate alone.  The bead's native partners sit in registers.
constexpr int kNlThreads = 256;
template <bool UNI, int L>
__global__ void __launch_bounds__(kNlThreads) k_nl(DevSys s) {
  const int k = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) / L);
  const int lane = threadIdx.x % L;
  const unsigned wl = threadIdx.x & 31;
  const unsigned gmask = group_mask<L>((int)wl);
  const unsigned below = (1u << wl) - 1u;
  if (k >= s.cell_start[s.cell_cap]) return;   // beads that were binned
  if (*s.flags & FLAG_NL_OVERFLOW) return;
  const float4 xi = s.xs[k];
  const int wi = __float_as_int(xi.w);
  const int i = wi >> 2, ti = wi & 3;
  const int m = s.mol_of[i];
  const MolGrid g = s.grid[m];
  const int lc = s.bead_cell[i] - g.base;
  const int nx = g.dims[0], ny = g.dims[1], nz = g.dims[2];
  const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
  const int z0 = max(cz - g.S, 0), z1 = min(cz + g.S, nz - 1);
  const int y0 = max(cy - g.S, 0), y1 = min(cy + g.S, ny - 1);
  const int x0 = max(cx - g.S, 0), x1 = min(cx + g.S, nx - 1);
  const float boxl = s.boxl;
  const bool wrap = g.wrap != 0;
  const float inv_cs = g.brute ? 0.0f : 1.0f / g.cs;
  const float r11 = s.rc2_nl_rep[1][1], r12 = s.rc2_nl_rep[1][2], r22 = s.rc2_nl_rep[2][2];
  const float rcm = s.rc_nl_rep_max * 1.0001f + 1.0e-3f;
  const float rcm2 = rcm * rcm;
  const int2 nrow = s.nat_row[i];
  int nat[kNatRegs];
#pragma unroll
  for (int q = 0; q < kNatRegs; ++q) nat[q] = q < nrow.y ? s.nat_j[nrow.x + q] : -1;
  const long long stride = s.nl_stride;
  unsigned short* row = s.nl_j + (long long)i * stride;  // partners relative to the molecule start
  const int mstart = s.mol[m].start;
  int cnt = 0;
  for (int z = z0; z <= z1; ++z) {
    const float dz = g.brute ? 0.0f : slab_dist(xi.z, g.lo[2] + z * g.cs, g.cs);
    if (dz * dz > rcm2) continue;
    for (int y = y0; y <= y1; ++y) {
      const float dy = g.brute ? 0.0f : slab_dist(xi.y, g.lo[1] + y * g.cs, g.cs);
      const float rem = rcm2 - dz * dz - dy * dy;
      if (rem < 0.0f) continue;
      int xa = x0, xb = x1;
      if (!g.brute) {
        // the chord only bounds the candidates (the exact predicate decides):
        // an approximate root and reciprocal, widened by 1e-3 A, keep it a
        // superset at a fraction of the cost of the exact operations
        const float w = __fmul_rn(rem, rsqrtf(fmaxf(rem, 1.0e-30f))) * 1.0001f + 1.0e-3f;
        xa = max(x0, cell_coord_fast(xi.x - w, g.lo[0], inv_cs, nx));
        xb = min(x1, cell_coord_fast(xi.x + w, g.lo[0], inv_cs, nx));
      }
      const int rowc = g.base + (z * ny + y) * nx;
      const int ja = s.cell_start[rowc + xa];
      const int jb = s.cell_start[rowc + xb] + s.cell_cnt[rowc + xb];
      for (int jc = ja; jc < jb; jc += L) {
        const int jj = jc + lane;
        bool pass = false;
        int j = 0;
        if (jj < jb) {
          const float4 xj = s.xs[jj];
          const int wj = __float_as_int(xj.w);
          j = wj >> 2;
          if (abs(j - i) > 2) {
            float dx = __fsub_rn(xj.x, xi.x), dy2 = __fsub_rn(xj.y, xi.y),
                  dz2 = __fsub_rn(xj.z, xi.z);
            if (wrap) min_image3(dx, dy2, dz2, boxl);
            pass = d2_exact(dx, dy2, dz2) < (UNI ? r11 : pick_type_pair(r11, r12, r22, ti, wj & 3));
            if (pass) {
              bool native = false;
#pragma unroll
              for (int q = 0; q < kNatRegs; ++q) native |= (nat[q] == j);
              for (int q = kNatRegs; q < nrow.y && !native; ++q) native = (s.nat_j[nrow.x + q] == j);
              pass = !native;
            }
          }
        }
        const unsigned msk = __ballot_sync(gmask, pass);
        if (pass) {
          const int pos = cnt + __popc(msk & below);
          if (pos < stride) row[pos] = (unsigned short)(j - mstart);
        }
        cnt += __popc(msk);
      }
    }
  }
  if (lane == 0) {
    s.nl_cnt[i] = cnt < stride ? cnt : (int)stride;
    if (cnt > stride) {
      atomicOr(s.flags, FLAG_NL_OVERFLOW);
      atomicMax(s.nl_maxrow, cnt);
    }
  }
}

// L lanes per bead (8: four beads per warp; 16 for molecules whose rows are
// long; 32: a warp per bead, for small contexts, where fewer than a wave of
// beads leaves the latency of each bead's rounds exposed): the pair list is
// the in-order compaction of the bead's neighbour-list row by the pair-list
// cut-off (sop.cu:835-920 semantics, host arithmetic of sop.cu:1737-1810).  Each lane takes 4
// consecutive entries per round (one 8-byte load, four independent gathers)
// and a scan across the group places the survivors; the attractive pair
// list is the same over the bead's attractive neighbour list.  The lists do
// not depend on L.
template <bool UNI, int L>
__global__ void __launch_bounds__(256, 5) k_pl(DevSys s, int koff) {  // 48 registers: 5 blocks per SM
  pdl_wait();
  pdl_release();
  const int wl = threadIdx.x & 31;
  const int lane = wl & (L - 1);
  const unsigned gmask = group_mask<L>(wl);
  // beads in chain order: the groups of a block gather from the same region
  // of a molecule, and the per-bead loads are coalesced
  const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) / L);
  if (i >= s.nlive) return;
  if (*s.flags & FLAG_NL_OVERFLOW) return;
  const int m = s.mol_of[i];
  if (!mol_listed(s, m, koff)) return;  // finished or stopped: keeps the lists of its last step
  const float4* X = xbuf(s, m, koff);
  const float4 xi = X[i];
  const int ti = type_of(xi);
  const float boxl = s.boxl;
  const bool wrap = s.grid[m].wrap != 0;  // from the neighbour-list build, with a cut-off of margin
  const float r11 = s.rc2_pl_rep[1][1], r12 = s.rc2_pl_rep[1][2], r22 = s.rc2_pl_rep[2][2];
  const unsigned below = (1u << wl) - 1u;  // lanes of the warp before this one
  const long long a = (long long)i * s.nl_stride;
  // rows hold partners relative to the molecule's first bead, 4 per 8 bytes
  const uint2* row4 = reinterpret_cast<const uint2*>(s.nl_j + a);
  unsigned short* out = s.pl_j + a;
  const int mstart = s.mol[m].start;
  const unsigned irel = (unsigned)(i - mstart);
  const unsigned self2 = irel | (irel << 16);  // two entries that name bead i
  const int cnt = s.nl_cnt[i];
  const int2 row = s.nat_row[i];
  const int acnt = s.nl_att_cnt[i];
  int k = 0;
  // each round works on entries loaded the round before (rows are read ahead)
  uint2 jn = make_uint2(self2, self2);
  if (4 * lane < cnt) jn = row4[lane];
  for (int e0 = 0; e0 < cnt; e0 += 4 * L) {
    const int e = e0 + 4 * lane;
    const uint2 jv = jn;
    jn = make_uint2(self2, self2);
    if (e + 4 * L < cnt) jn = row4[(e0 >> 2) + L + lane];
    const int jq[4] = {mstart + (int)(jv.x & 0xffffu),
                       e + 1 < cnt ? mstart + (int)(jv.x >> 16) : i,
                       e + 2 < cnt ? mstart + (int)(jv.y & 0xffffu) : i,
                       e + 3 < cnt ? mstart + (int)(jv.y >> 16) : i};
    unsigned pb = 0;
    int c = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 xj = X[jq[q]];
      float dx = __fsub_rn(xj.x, xi.x), dy = __fsub_rn(xj.y, xi.y),
            dz = __fsub_rn(xj.z, xi.z);
      if (wrap) min_image3(dx, dy, dz, boxl);
      const bool p = (e + q < cnt) &&
                     d2_exact(dx, dy, dz) < (UNI ? r11 : pick_type_pair(r11, r12, r22, ti, type_of(xj)));
      pb |= (p ? 1u : 0u) << q;
      c += p ? 1 : 0;
    }
    int incl = c;
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
      const int t = __shfl_up_sync(gmask, incl, o, L);
      if (lane >= o) incl += t;
    }
    int pos = k + incl - c;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (pb & (1u << q)) out[pos++] = (unsigned short)(jq[q] - mstart);
    k += __shfl_sync(gmask, incl, L - 1, L);
  }
  if (lane == 0) s.pl_cnt[i] = k;
  int ka = 0;
  for (int e0 = 0; e0 < acnt; e0 += L) {
    const int e = e0 + lane;
    bool pass = false;
    int j = 0;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e < acnt) {
      const int idx = s.nl_att_e[row.x + e];
      // the contact's partner, cut-off and parameters in one round of loads
      j = s.nat_j[idx];
      const float rc2 = s.nat_rc2[idx].y;
      q = s.nat_par[idx];
      const float4 xj = X[j];
      float dx = __fsub_rn(xj.x, xi.x), dy = __fsub_rn(xj.y, xi.y),
            dz = __fsub_rn(xj.z, xi.z);
      if (wrap) min_image3(dx, dy, dz, boxl);
      pass = d2_exact(dx, dy, dz) < rc2;
    }
    const unsigned mask = __ballot_sync(gmask, pass) & gmask;
    if (pass) s.pl_att[row.x + ka + __popc(mask & below)] = make_float4(__int_as_float(j), q.x, q.y, q.z);
    ka += __popc(mask);
  }
  if (lane == 0) s.pl_att_cnt[i] = ka;
}

// ------------------------------------------------------------ host side
static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Launch sequence of an exclusive scan of n ints (in -> out[0..n]).
void launch_scan(const int* in, long long n, int* out, int* block_sums, cudaStream_t st) {
  unsigned nb = cdiv(n > 0 ? n : 1, kScanTile);
  k_scan_reduce<<<nb, kScanThreads, 0, st>>>(in, n, block_sums);
  k_scan_top<<<1, 1024, 0, st>>>(block_sums, (int)nb);
  k_scan_apply<<<nb, kScanThreads, 0, st>>>(in, n, block_sums, out);
}

long long scan_block_sums_needed(long long n) { return cdiv(n > 0 ? n : 1, kScanTile) + 1; }

struct NLScratch {
  int* ncell;        // per molecule
  int* block_sums;
  int* cells_total;  // one int: cells in use
};

// Cell binning of the molecules a rebuild at koff covers: the cell order the
// neighbour-list build walks, and each molecule's grid flags (wrap: whether
// the minimum image can matter), which the step and pair-list kernels read;
// att = 1 also refreshes the attractive neighbour lists.
static void launch_binning(const DevSys& s, const NLScratch& w, int koff, int att, cudaStream_t st) {
  if (s.nlive <= kWideListBeads && s.cell_cap <= kBinSmallCells) {
    k_bin_small<<<1, kBinThreads, 0, st>>>(s, w.ncell, w.cells_total, koff, att);
    return;
  }
  const int T = 256;
  k_bbox_reset<<<cdiv(s.nmol, T), T, 0, st>>>(s);
  k_bbox<<<cdiv(s.nlive, T), T, 0, st>>>(s, koff);
  k_grid<<<cdiv(s.nmol, T), T, 0, st>>>(s, w.ncell, koff);
  k_grid_base<<<1, 1024, 0, st>>>(s, w.ncell, w.cells_total);
  cudaMemsetAsync(s.cell_cnt, 0, sizeof(int) * (size_t)s.cell_cap, st);
  k_assign<<<cdiv(s.nlive, T), T, 0, st>>>(s, koff, att);
  launch_scan(s.cell_cnt, s.cell_cap, s.cell_start, w.block_sums, st);
  k_scatter<<<cdiv(s.nlive, T), T, 0, st>>>(s);
  k_cellsort<<<cdiv(s.cell_cap, T), T, 0, st>>>(s, w.cells_total);
  k_stage_xs<<<cdiv(s.nlive, T), T, 0, st>>>(s, koff);
}

// Full neighbour-list rebuild from the coordinates at step mol_step + koff.
void launch_nl_rebuild(const DevSys& s, const NLScratch& w, int koff, cudaStream_t st) {
  const int T = kNlThreads;
  launch_binning(s, w, koff, 1, st);
  const bool wide = s.nlive <= kWideListBeads;
  const unsigned grid = cdiv((long long)s.nlive * (wide ? 32 : 8), T);
  if (s.uniform_type) {
    if (wide) k_nl<true, 32><<<grid, T, 0, st>>>(s);
    else k_nl<true, 8><<<grid, T, 0, st>>>(s);
  } else {
    if (wide) k_nl<false, 32><<<grid, T, 0, st>>>(s);
    else k_nl<false, 8><<<grid, T, 0, st>>>(s);
  }
}

// The binning alone, every list untouched: molecules that arrive with their
// lists (restored from a checkpoint) get grid flags from their own
// coordinates, which the step and pair-list kernels need.  The cell order
// itself decides no result.
void launch_rebin(const DevSys& s, const NLScratch& w, cudaStream_t st) {
  launch_binning(s, w, 0, 0, st);
}

void launch_pl_rebuild(const DevSys& s, int koff, cudaStream_t st) {
  const int T = 256;
  const int L = s.nlive <= kWideListBeads ? 32 : (s.long_rows ? 16 : 8);
  const unsigned grid = cdiv((long long)s.nlive * L, T);
  if (s.uniform_type)
    launch_pdl(L == 32 ? k_pl<true, 32> : L == 16 ? k_pl<true, 16> : k_pl<true, 8>, grid, T, st, s,
               koff);
  else
    launch_pdl(L == 32 ? k_pl<false, 32> : L == 16 ? k_pl<false, 16> : k_pl<false, 8>, grid, T, st,
               s, koff);
}

}  // namespace sop
