// The per-step hot path: forces (FENE, i,i+2 soft sphere, native LJ 12-6,
// non-native repulsion), the Philox noise force and the underdamped Langevin
// update, fused into one kernel per step.
//
// The reference runs per step underdamped_iteration_kernel (sop.cu:421-447),
// clear_forces + rand_kernel + four force kernels with float atomics
// (energy.cu:54-167, 228-584) and update_velocities_kernel (sop.cu:450-462).
// Here a group of G lanes owns a bead (beads in chain order: neighbouring
// groups gather from the same region of a molecule, and the per-bead loads
// are coalesced): it sums the bead's force
// over its own full rows (every pair is stored for both beads) in an order
// that does not depend on G, then one thread per bead adds the noise and
// updates velocity and coordinates.  No atomics.
//
// Step bookkeeping: kernel K_n computes f_n = F(x_n) + noise(n), then
// v_n = a3 incr_n + a4 f_n, then the look-ahead incr_{n+1} = a1 v_n + a2 f_n
// and x_{n+1} = x_n + incr_{n+1}.  This is the reference's order
// (incr, positions, forces, velocities) regrouped so one kernel per step
// suffices.  x_n lives in buffer n & 1, so neither the host nor a graph has
// to track parity, and every molecule may sit at its own step.
#include <algorithm>

#include "sop_dev.cuh"
#include "../../include/sop_gpu.h"

namespace sop {

constexpr int kV = 16;  // virtual lanes of the fixed force-summation order

constexpr int kStepThreads = 128;  // small blocks: a finished block frees its SM slot sooner

// Blocks per SM each lane-group width is compiled for (a register cap).
template <int G>
struct StepBlocks {
  static constexpr int value = G == 4 ? 10 : (G == 8 ? 12 : (G == 16 ? 8 : 2));
};

// Every rounding of the per-entry arithmetic and of the accumulation is
// written out (one rounding per operation), so the compiler cannot contract
// it differently in different instantiations: the sums are then the same
// bits for every lane-group width.
__device__ __forceinline__ void acc3(float& ax, float& ay, float& az, float c, float dx, float dy,
                                     float dz) {
  ax = __fmaf_rn(c, dx, ax);
  ay = __fmaf_rn(c, dy, ay);
  az = __fmaf_rn(c, dz, az);
}

__device__ __forceinline__ float d2_plain(float dx, float dy, float dz) {
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Force coefficient of one bonded / angle / native entry (type 0 / 1 / 2):
// the reference kernels' formulas, with the compensated d^2 - r0^2 wherever
// a difference from the native distance enters.
__device__ __forceinline__ float small_coeff(const DevSys& s, int type, float dx, float dy, float dz,
                                             float lx, float ly, float lz, float r0, float eps,
                                             bool& fene_bad) {
  const float d2 = d2_plain(dx, dy, dz);
  if (type == 0) {
    // FENE: force on i = +k dev / (r (1 - dev^2/R0^2)) * d  (energy.cu:252-271);
    // dev carries the compensated d^2 - r0^2, so approximate reciprocals
    // (a few ulps) keep the term well inside the force tolerance
    const float r = __fmul_rn(d2, rsqrtf(d2));
    const float dev = __fmul_rn(d2_minus_r02(dx, dy, dz, lx, ly, lz, r0),
                                __fdividef(1.0f, __fadd_rn(r, r0)));
    const float w = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(dev, dev), s.inv_R0sq));
    fene_bad |= !(fabsf(dev) < s.R0);
    return __fmul_rn(__fmul_rn(s.k_bnd, dev), __fdividef(1.0f, __fmul_rn(r, w)));
  }
  if (type == 1) {
    // i,i+2 soft sphere: force on i = -6 eps sigma^6 / d^8 * d  (energy.cu:335-360)
    const float inv = __fdividef(1.0f, d2);
    const float inv2 = __fmul_rn(inv, inv);
    return __fmul_rn(-s.f_ss, __fmul_rn(inv2, inv2));
  }
  // native LJ 12-6 (energy.cu:468-507): co1 = -12 eps / d^2 (s^6 - s^3),
  // s = r0^2 / d^2, as -12 eps / d^2 s^3 (s - 1)(s^2 + s + 1) with
  // s - 1 = -(d^2 - r0^2) / d^2; pairs with d^2 <= 1e-7 r0^2 are skipped.
  const float r02 = __fmul_rn(r0, r0);
  const float inv = __fdividef(1.0f, d2);
  const float sr = __fmul_rn(r02, inv);
  const float sm1 = __fmul_rn(-d2_minus_r02(dx, dy, dz, lx, ly, lz, r0), inv);
  const float s3 = __fmul_rn(__fmul_rn(sr, sr), sr);
  const float poly = __fadd_rn(__fadd_rn(__fmul_rn(sr, sr), sr), 1.0f);
  const float c =
      __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(-12.0f, eps), inv), __fmul_rn(s3, sm1)), poly);
  return d2 > __fmul_rn(1.0e-7f, r02) ? c : 0.0f;
}

// STEP = false: force evaluation only at step mol_step + koff (velocities kept),
// followed by the look-ahead; used after set-up and state uploads.
// Marker bits in the w of a bead's force sum (0: not summed this step).
constexpr int kSummed = 1;
constexpr int kFeneBad = 2;   // a bond at or past R0
constexpr int kOddStep = 4;   // the step is odd: coordinates in buffer 1

template <bool STEP>
__device__ __forceinline__ void finish_bead(const DevSys& s, int b, int m, float4 fs, int koff);

// Coordinate sources of the force sum: the molecule's coordinate buffer in
// global memory, or the block's window of it staged in shared memory (bead j
// at xw[j - off]).  The arithmetic is the same either way, so are the bits.
struct GlobalX {
  const float4* __restrict__ p;
  __device__ __forceinline__ float4 operator()(int j) const { return p[j]; }
};
struct WindowX {
  const float4* p;  // shared memory
  int off;
  __device__ __forceinline__ float4 operator()(int j) const { return p[j - off]; }
};

// The conservative force on bead i, summed by the G lanes of its group over
// its rows (bonds, angles, native pair list, repulsive pair list) into the
// lane's kC virtual-lane accumulators, reduced to lane 0 of the group.
// Forces are summed in a fixed order whatever G is: entry e of a row
// accumulates into virtual lane e % kV (in increasing e), and the kV partial
// sums combine in one fixed binary tree (pairs v, v + kV/2, then v, v + kV/4,
// ...).  Each physical lane holds kC = kV / G virtual lanes and does the
// upper tree levels locally, the rest by shuffles.  So every G gives
// bit-identical forces, and G is free to tune per context.
template <int G, bool UNI, class XS>
__device__ __forceinline__ void bead_force(const DevSys& s, const XS& X, int i, int m1, int lane,
                                           int2 br, int2 ar, int abase, int acnt, int rcnt,
                                           float& fx, float& fy, float& fz, bool& fene_bad) {
  constexpr int kC = kV / G;
  float ax[kC], ay[kC], az[kC];
#pragma unroll
  for (int c = 0; c < kC; ++c) ax[c] = ay[c] = az[c] = 0.f;
  const unsigned gmask = (G == 32) ? 0xffffffffu
                                   : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const float4 xi = X(i);
  const float boxl = s.boxl;
  // 0 when no pair of the molecule can reach boxl/4 (from its last binning,
  // with a cut-off of margin): the minimum image is then the identity and
  // its test is skipped
  const bool wrap = s.grid[m1].wrap != 0;
  const long long rbase = (long long)i * s.nl_stride;

  // Bonded, angle and native terms share one index space [bonds | angles |
  // natives]; a bead has a handful of them, usually one pass.
  const int nba = br.y + ar.y;
  const int nsmall = nba + acnt;
  for (int base = 0; base < nsmall; base += kV) {
#pragma unroll
    for (int c = 0; c < kC; ++c) {
      const int e = base + lane + c * G;
      if (e >= nsmall) continue;
      int j, t;
      float r0 = 0.f, eps = 0.f;
      if (e < br.y) {
        j = s.bond_j[br.x + e];
        r0 = s.bond_r0[br.x + e];
        t = 0;
      } else if (e < nba) {
        j = s.ang_j[ar.x + e - br.y];
        t = 1;
      } else {
        const float4 q = s.pl_att[abase + e - nba];
        j = __float_as_int(q.x);
        r0 = q.y;
        eps = q.z;
        t = 2;
      }
      const float4 xj = X(j);
      float lx, ly, lz;
      float dx = diff_exact(xj.x, xi.x, lx), dy = diff_exact(xj.y, xi.y, ly),
            dz = diff_exact(xj.z, xi.z, lz);
      if (wrap) min_image3(dx, dy, dz, boxl);
      const float cc = small_coeff(s, t, dx, dy, dz, lx, ly, lz, r0, eps, fene_bad);
      acc3(ax[c], ay[c], az[c], cc, dx, dy, dz);
    }
  }

  // Non-native repulsion (energy.cu:536-581): co1 = -6 eps / d^2 (2 (s/r)^12 +
  // (s/r)^6) [rep6: -6 eps / d^2 (s/r)^6]; pairs with d^2 <= 1e-7 sigma are
  // skipped.  kC loads in flight per lane per chunk of kV entries.  A system
  // of one bead type (UNI) uses its sigma as a constant.
  const int ti = type_of(xi);
  const float g11 = s.sig2[1][1], g12 = s.sig2[1][2], g22 = s.sig2[2][2];
  const float t11 = s.rep_tol[1][1], t12 = s.rep_tol[1][2], t22 = s.rep_tol[2][2];
  const float ce = -6.0f * s.eps_rep;
  const float two = s.rep6 ? 0.0f : 2.0f;
  const float q4 = 0.25f * boxl;
  // pair-list partners are stored relative to the molecule's first bead
  const unsigned short* __restrict__ prow = s.pl_j + rbase;
  const int jbase = s.mol[m1].start;
  for (int base = 0; base < rcnt; base += kV) {
    int jj[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
      const int e = base + lane + c * G;
      jj[c] = e < rcnt ? jbase + (int)prow[e] : i;
    }
    float4 xx[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) xx[c] = X(jj[c]);
#pragma unroll
    for (int c = 0; c < kC; ++c) {
      // past the row end xx[c] is bead i itself: d2 = 0 fails the tolerance
      // test and contributes exactly 0, so no branch is needed
      float dx = __fsub_rn(xx[c].x, xi.x), dy = __fsub_rn(xx[c].y, xi.y),
            dz = __fsub_rn(xx[c].z, xi.z);
      // |dx| + |dy| + |dz| bounds every component: one test for the rare wrap
      if (wrap && fabsf(dx) + fabsf(dy) + fabsf(dz) > q4) min_image3(dx, dy, dz, boxl);
      const float d2 = d2_plain(dx, dy, dz);
      float sg2 = g11, tol = t11;
      if (!UNI) {
        const int tj = type_of(xx[c]);
        sg2 = pick_type_pair(g11, g12, g22, ti, tj);
        tol = pick_type_pair(t11, t12, t22, ti, tj);
      }
      const float inv = __fdividef(1.0f, d2);
      const float u = __fmul_rn(sg2, inv);
      const float u3 = __fmul_rn(__fmul_rn(u, u), u);
      const float cc = (d2 > tol) ? __fmul_rn(__fmul_rn(__fmul_rn(ce, inv), u3), __fmaf_rn(two, u3, 1.0f))
                                  : 0.0f;
      acc3(ax[c], ay[c], az[c], cc, dx, dy, dz);
    }
  }
  // upper levels of the fixed tree inside the lane, lower levels by shuffles
#pragma unroll
  for (int off = kV / 2; off >= G; off >>= 1) {
    const int oc = off / G;
#pragma unroll
    for (int c = 0; c < kC; ++c)
      if (c < oc) {
        ax[c] = __fadd_rn(ax[c], ax[c + oc]);
        ay[c] = __fadd_rn(ay[c], ay[c + oc]);
        az[c] = __fadd_rn(az[c], az[c + oc]);
      }
  }
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) {
    ax[0] = __fadd_rn(ax[0], __shfl_xor_sync(gmask, ax[0], off));
    ay[0] = __fadd_rn(ay[0], __shfl_xor_sync(gmask, ay[0], off));
    az[0] = __fadd_rn(az[0], __shfl_xor_sync(gmask, az[0], off));
  }
  fene_bad = __any_sync(gmask, fene_bad);
  fx = ax[0];
  fy = ay[0];
  fz = az[0];
}

// SPLIT = false: one kernel -- the groups' sums go through shared memory to
// one thread per bead, which completes the step (finish_bead).  SPLIT = true:
// the sums go to s.fsum and k_finish completes the step in a second launch
// (no block barrier, coalesced state access; faster for large contexts).
// Both complete a bead with the same finish_bead, so the results are the
// same bits.
//
// WIN = true: the block first stages the coordinates of the molecules its
// beads belong to -- the contiguous bead range from the first bead's
// molecule start to the last bead's molecule end, every bead from its own
// molecule's current buffer -- into dynamic shared memory (up to wcap beads),
// with coalesced loads; every partner of a bead lies in its own molecule, so
// all gathers of the force sum then hit shared memory instead of L2.  A block
// whose range exceeds wcap (or holds a free slot) gathers from global memory.
// What a lane group needs about its bead slot b1 for step mol_step + STEP +
// koff: the bead (-1: nothing to do -- a free slot, an inactive, failed,
// finished or not yet started molecule), its molecule, the step and its row
// descriptors.
struct BeadSlot {
  int i = -1, m1 = -1;
  long long n = 0;
  int2 br = make_int2(0, 0), ar = make_int2(0, 0);
  int abase = 0, acnt = 0, rcnt = 0;
};

template <bool STEP>
__device__ __forceinline__ BeadSlot bead_slot(const DevSys& s, int b1, int koff) {
  BeadSlot q;
  const bool live = b1 < s.nlive && !(*s.flags & FLAG_NL_OVERFLOW);
  q.m1 = live ? s.mol_of[b1] : -1;  // -1: a free slot
  // Row descriptors, loaded beside the molecule's state rather than after
  // its test: they do not depend on it.
  if (live) {
    q.br = s.bond_row[b1];
    q.ar = s.ang_row[b1];
    q.abase = s.nat_row[b1].x;
    q.acnt = s.pl_att_cnt[b1];
    q.rcnt = s.pl_cnt[b1];
  }
  if (q.m1 >= 0) {
    const MolConst& mc = s.mol[q.m1];
    q.n = s.mol_step[q.m1] + (STEP ? 1 : 0) + koff;
    // n < 0: a molecule admitted to a running context whose step 0 comes later
    // in this block; n > nsteps: finished
    if (mc.active && s.mol_status[q.m1] == 0 && q.n >= 0 &&
        !(STEP && mc.nsteps >= 0 && q.n > mc.nsteps))
      q.i = b1;
  }
  return q;
}

// The force sum's w: the marker bits of finish_bead (summed, a bond past R0,
// the parity of the step, which selects the coordinate buffers).
__device__ __forceinline__ float4 marked_sum(float fx, float fy, float fz, bool fene_bad,
                                             long long n) {
  return make_float4(fx, fy, fz,
                     __int_as_float(kSummed | (fene_bad ? kFeneBad : 0) |
                                    ((int)(n & 1) ? kOddStep : 0)));
}

template <int G, bool STEP, bool UNI, bool SPLIT, bool WIN>
__global__ void __launch_bounds__(kStepThreads, StepBlocks<G>::value) k_step(DevSys s, int koff,
                                                                            int wcap) {
  constexpr int BPB = kStepThreads / G;  // beads per block
  extern __shared__ float4 xwin[];
  __shared__ int win_lo, win_n;          // window start bead and length (-1: none)
  pdl_wait();
  pdl_release();
  const int slot = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const int b1 = blockIdx.x * BPB + slot;
  const BeadSlot q = bead_slot<STEP>(s, b1, koff);
  const int i = q.i, m1 = q.m1;
  const long long n = q.n;
  if (WIN) {
    if (threadIdx.x == 0) {
      int lo = 0, len = -1;
      const int b0 = blockIdx.x * BPB;
      const int bl = min(b0 + BPB, s.nlive) - 1;
      if (b0 <= bl && !(*s.flags & FLAG_NL_OVERFLOW)) {
        const int m0 = s.mol_of[b0], ml = s.mol_of[bl];
        if (m0 >= 0 && ml >= 0) {
          lo = s.mol[m0].start;
          const int hi = s.mol[ml].start + s.mol[ml].n;
          if (hi - lo <= wcap) len = hi - lo;
        }
      }
      win_lo = lo;
      win_n = len;
    }
    __syncthreads();
    const int lo = win_lo, len = win_n;
    for (int k = threadIdx.x; k < len; k += kStepThreads) {
      const int b = lo + k;
      const int m = s.mol_of[b];
      const int par = m >= 0 ? (int)((s.mol_step[m] + (STEP ? 1 : 0) + koff) & 1) : 0;
      xwin[k] = s.x[par][b];
    }
    __syncthreads();
  }
  float fx = 0.f, fy = 0.f, fz = 0.f;
  bool fene_bad = false;
  if (i >= 0) {  // uniform over the lane group
    if (WIN && win_n >= 0) {
      bead_force<G, UNI>(s, WindowX{xwin, win_lo}, i, m1, lane, q.br, q.ar, q.abase, q.acnt,
                         q.rcnt, fx, fy, fz, fene_bad);
    } else {
      bead_force<G, UNI>(s, GlobalX{s.x[(int)(n & 1)]}, i, m1, lane, q.br, q.ar, q.abase, q.acnt,
                         q.rcnt, fx, fy, fz, fene_bad);
    }
  }
  const float4 sum = marked_sum(fx, fy, fz, fene_bad, n);
  if (SPLIT) {
    // the group's sum, marked for k_finish (which completes the step)
    if (i >= 0 && lane == 0) s.fsum[i] = sum;
    return;
  }
  __shared__ float4 fsum[BPB];          // the slots' sums (w as in s.fsum)
  __shared__ int bead[BPB];             // bead of each slot, -1: nothing to do
  if (lane == 0) {
    fsum[slot] = sum;
    bead[slot] = i;
  }
  __syncthreads();
  if (threadIdx.x >= BPB) return;
  const int b = bead[threadIdx.x];
  if (b < 0) return;
  finish_bead<STEP>(s, b, s.mol_of[b], fsum[threadIdx.x], koff);
}

// What completing bead b (of molecule m) at step mol_step + STEP + koff needs
// besides its force sum: its state (coordinates from buffer cur, the step's
// parity) and its noise.  None of it is written by the force kernel of the
// same step.
struct BeadState {
  MolConst mc;
  long long nb;
  float4 vi, inc, xo, pi;
  float3 z;
};

template <bool STEP>
__device__ __forceinline__ void load_bead_state(const DevSys& s, int b, int m, int koff, int cur,
                                                BeadState& t) {
  t.mc = s.mol[m];
  t.nb = s.mol_step[m] + (STEP ? 1 : 0) + koff;
  t.vi = s.v[b];
  t.inc = s.incr[b];
  t.xo = s.x[cur][b];
  t.pi = s.p[cur][b];
  if (s.use_noise) {
    const float4 q = s.noise[b];
    t.z = make_float3(q.x, q.y, q.z);
  } else {
    t.z = noise3((unsigned)(b - t.mc.start), t.nb, t.mc.traj, s.seed_lo, s.seed_hi);
  }
}

// Completes bead b from its conservative force sum fs, whose w holds the
// marker bits k_step set: noise, status, velocity and the look-ahead
// position update (sop.cu:421-462, energy.cu:588-604).  Every rounding is
// written out.
template <bool STEP>
__device__ __forceinline__ void complete_bead(const DevSys& s, int b, int m, float4 fs, int cur,
                                              const BeadState& t) {
  const int w = __float_as_int(fs.w);
  const MolConst& mc = t.mc;
  float4 vi = t.vi;
  float4 inc = t.inc;
  const float4 xo = t.xo;
  const float4 pi = t.pi;
  const float3 z = t.z;
  const float fxx = __fmaf_rn(mc.sigma_f, z.x, fs.x);
  const float fyy = __fmaf_rn(mc.sigma_f, z.y, fs.y);
  const float fzz = __fmaf_rn(mc.sigma_f, z.z, fs.z);
  int st = 0;
  if (w & kFeneBad) st |= SOP_MOL_FENE_RANGE;
  if (!(isfinite(fxx) && isfinite(fyy) && isfinite(fzz))) st |= SOP_MOL_NONFINITE;
  if (st) atomicOr(s.mol_status + m, st);
  s.f[b] = make_float4(fxx, fyy, fzz, 0.f);
  // step 0 is the initial force evaluation (sop.cu:180-186): velocities stay
  if (STEP && t.nb > 0 && !mc.t_zero) {
    vi = make_float4(__fmaf_rn(mc.a3, inc.x, __fmul_rn(mc.a4, fxx)),
                     __fmaf_rn(mc.a3, inc.y, __fmul_rn(mc.a4, fyy)),
                     __fmaf_rn(mc.a3, inc.z, __fmul_rn(mc.a4, fzz)), 0.f);
    s.v[b] = vi;
  }
  inc = make_float4(__fmaf_rn(mc.a1, vi.x, __fmul_rn(mc.a2, fxx)),
                    __fmaf_rn(mc.a1, vi.y, __fmul_rn(mc.a2, fyy)),
                    __fmaf_rn(mc.a1, vi.z, __fmul_rn(mc.a2, fzz)), 0.f);
  s.incr[b] = inc;
  s.x[cur ^ 1][b] = make_float4(__fadd_rn(xo.x, inc.x), __fadd_rn(xo.y, inc.y),
                                __fadd_rn(xo.z, inc.z), xo.w);
  const float boxl = s.boxl;
  s.p[cur ^ 1][b] = make_float4(min_image(__fadd_rn(pi.x, inc.x), boxl),
                                min_image(__fadd_rn(pi.y, inc.y), boxl),
                                min_image(__fadd_rn(pi.z, inc.z), boxl), 0.f);
}

// Completes bead b (of molecule m) from its force sum fs; the step is the
// molecule's mol_step + STEP + koff, as in k_step, and its parity (which
// selects the coordinate buffers) is marked in fs.w.
template <bool STEP>
__device__ __forceinline__ void finish_bead(const DevSys& s, int b, int m, float4 fs, int koff) {
  const int cur = (__float_as_int(fs.w) & kOddStep) ? 1 : 0;
  BeadState t;
  load_bead_state<STEP>(s, b, m, koff, cur, t);
  complete_bead<STEP>(s, b, m, fs, cur, t);
}

// Second kernel of the split step: completes every bead k_step summed
// (thread per bead, bead order, so every state access is coalesced).  The
// bead's state and noise do not depend on the force kernel this kernel
// follows, so they load (and the noise is drawn) before the wait on it:
// with programmatic dependent launch that work overlaps the force kernel's
// last blocks.  The force kernel marked the same parity (both read the
// molecule's step, which only the step advance changes).
template <bool STEP>
__global__ void __launch_bounds__(256, 6) k_finish(DevSys s, int koff) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= s.nlive) return;
  const int m = s.mol_of[b];
  if (m < 0) return;  // a free slot: nothing was summed
  // a molecule k_step skips for good (inactive, not started or finished:
  // the tests of bead_slot on values no kernel of this step writes) has
  // nothing to finish; a stopped one is caught by its unmarked sum below
  // (its status bits may be set by this very kernel)
  const MolConst& mc = s.mol[m];
  const long long n = s.mol_step[m] + (STEP ? 1 : 0) + koff;
  if (!mc.active || n < 0 || (STEP && mc.nsteps >= 0 && n > mc.nsteps)) return;
  const int cur = (int)(n & 1);
  BeadState t;
  load_bead_state<STEP>(s, b, m, koff, cur, t);
  pdl_wait();
  pdl_release();
  const float4 fs = s.fsum[b];
  if (__float_as_int(fs.w) == 0) return;  // not summed this step
  s.fsum[b].w = 0.0f;
  complete_bead<STEP>(s, b, m, fs, cur, t);
}

// ------------------------------------------------------------ tiled form
// Per-molecule tiles with per-tile shapes: each block takes one tile -- the
// beads [t.x, t.y) of a single molecule (at most 128 / G of them) -- with
// t.z lanes per bead (4 or 8) and t.w = 1 for the two-kernel form (the sum
// goes to fsum for k_finish) or 0 (completed in the block).  The host builds
// the tiles so that every molecule of a size bucket gets the shape the
// autotuner chose for that bucket; one launch covers every bucket.  The
// per-bead code is k_step's, so the bits are the same.
template <int G, bool STEP, bool UNI>
__device__ __forceinline__ void tile_body(const DevSys& s, int koff, int4 t, float4* fsum,
                                          int* bead) {
  constexpr int BPB = kStepThreads / G;
  const int slot = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const int b1 = t.x + slot;
  BeadSlot q;
  if (b1 < t.y) q = bead_slot<STEP>(s, b1, koff);
  float fx = 0.f, fy = 0.f, fz = 0.f;
  bool fene_bad = false;
  if (q.i >= 0)
    bead_force<G, UNI>(s, GlobalX{s.x[(int)(q.n & 1)]}, q.i, q.m1, lane, q.br, q.ar, q.abase,
                       q.acnt, q.rcnt, fx, fy, fz, fene_bad);
  const float4 sum = marked_sum(fx, fy, fz, fene_bad, q.n);
  if (t.w) {
    if (q.i >= 0 && lane == 0) s.fsum[q.i] = sum;
    return;
  }
  if (lane == 0) {
    fsum[slot] = sum;
    bead[slot] = q.i;
  }
  __syncthreads();
  if (threadIdx.x >= BPB) return;
  const int b = bead[threadIdx.x];
  if (b >= 0) finish_bead<STEP>(s, b, s.mol_of[b], fsum[threadIdx.x], koff);
}

template <bool STEP, bool UNI>
__global__ void __launch_bounds__(kStepThreads, StepBlocks<4>::value)
    k_step_tiles(DevSys s, int koff, const int4* __restrict__ tiles) {
  __shared__ float4 fsum[kStepThreads / 4];
  __shared__ int bead[kStepThreads / 4];
  pdl_wait();
  pdl_release();
  const int4 t = tiles[blockIdx.x];   // uniform over the block
  if (t.z == 8) tile_body<8, STEP, UNI>(s, koff, t, fsum, bead);
  else tile_body<4, STEP, UNI>(s, koff, t, fsum, bead);
}

// ------------------------------------------------------ persistent form
// Every step of a run of steps with no list rebuild in between, in one
// cooperative launch: each block owns bead chunks (grid-stride) and completes
// them step after step, with a device-wide barrier between steps (x_{n+1} of
// every bead is written before any bead's force of step n+1 reads it).  The
// per-bead code is k_step's one-kernel form, so the bits are the same.
//
// The barrier: bar[0] counts the blocks that arrived, bar[1] is the
// generation.  The last block to arrive resets the count and advances the
// generation; the others wait for it with a time limit, after which they set
// FLAG_BARRIER_TIMEOUT and the whole launch returns (the host reports the
// context as failed and clears the count).  `expected` is the number of
// arrivals that complete the barrier: gridDim.x, or more for the check that
// makes the wait run out on purpose.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Called by every thread of the block; returns false on a timed-out wait.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned expected, unsigned& gen,
                                             unsigned long long limit_ns, int* flags) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    __threadfence();
    if (atomicAdd(&bar[0], 1u) + 1u == expected) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_gpu(&bar[1]) == gen) {
        if (global_ns() - t0 > limit_ns) {
          good = 0;
          atomicOr(flags, FLAG_BARRIER_TIMEOUT);
          break;
        }
        __nanosleep(100);
      }
      __threadfence();
    }
    ++gen;
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <int G, bool STEP, bool UNI>
__global__ void __launch_bounds__(kStepThreads, StepBlocks<G>::value)
    k_step_persist(DevSys s, int koff0, int count,
                                                               unsigned* bar, unsigned expected,
                                                               unsigned long long limit_ns) {
  constexpr int BPB = kStepThreads / G;
  __shared__ float4 fsum[BPB];
  __shared__ int bead[BPB];
  __shared__ unsigned gen0;
  pdl_wait();
  pdl_release();
  // every block reads the generation before it first arrives, so all agree
  if (threadIdx.x == 0) gen0 = ld_acquire_gpu(&bar[1]);
  __syncthreads();
  unsigned gen = gen0;
  const int slot = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const int nchunks = (s.nlive + BPB - 1) / BPB;
  for (int k = 0; k < count; ++k) {
    if (k > 0 && !grid_barrier(bar, expected, gen, limit_ns, s.flags)) return;
    // steps advance the block offset; force-only evaluations (STEP = false,
    // repeated for timing) recompute the same step, which keeps them idempotent
    const int koff = STEP ? koff0 + k : koff0;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
      const BeadSlot q = bead_slot<STEP>(s, c * BPB + slot, koff);
      float fx = 0.f, fy = 0.f, fz = 0.f;
      bool fene_bad = false;
      if (q.i >= 0)
        bead_force<G, UNI>(s, GlobalX{s.x[(int)(q.n & 1)]}, q.i, q.m1, lane, q.br, q.ar, q.abase,
                           q.acnt, q.rcnt, fx, fy, fz, fene_bad);
      if (lane == 0) {
        fsum[slot] = marked_sum(fx, fy, fz, fene_bad, q.n);
        bead[slot] = q.i;
      }
      __syncthreads();
      if (threadIdx.x < BPB) {
        const int b = bead[threadIdx.x];
        if (b >= 0) finish_bead<STEP>(s, b, s.mol_of[b], fsum[threadIdx.x], koff);
      }
      __syncthreads();
    }
  }
}

// One block of 1,024 threads runs every step between two list rebuilds:
// for contexts of a few hundred beads, where each step is a short chain of
// dependent loads and a kernel boundary (even overlapped by programmatic
// dependent launch) costs as much as the step.  Steps are separated by
// block barriers; the per-bead code is k_step's, so the bits are the same.
constexpr int kBlockFormThreads = 1024;
template <int G, bool STEP, bool UNI>
__global__ void __launch_bounds__(kBlockFormThreads, 1) k_step_block(DevSys s, int koff0, int count) {
  constexpr int BPB = kBlockFormThreads / G;
  __shared__ float4 fsum[BPB];
  __shared__ int bead[BPB];
  pdl_wait();
  pdl_release();
  const int slot = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const int nchunks = (s.nlive + BPB - 1) / BPB;
  for (int k = 0; k < count; ++k) {
    // force-only evaluations (STEP = false, repeated for timing) recompute
    // the same step, which keeps them idempotent
    const int koff = STEP ? koff0 + k : koff0;
    for (int c = 0; c < nchunks; ++c) {
      const BeadSlot q = bead_slot<STEP>(s, c * BPB + slot, koff);
      float fx = 0.f, fy = 0.f, fz = 0.f;
      bool fene_bad = false;
      if (q.i >= 0)
        bead_force<G, UNI>(s, GlobalX{s.x[(int)(q.n & 1)]}, q.i, q.m1, lane, q.br, q.ar, q.abase,
                           q.acnt, q.rcnt, fx, fy, fz, fene_bad);
      if (lane == 0) {
        fsum[slot] = marked_sum(fx, fy, fz, fene_bad, q.n);
        bead[slot] = q.i;
      }
      __syncthreads();
      if (threadIdx.x < BPB) {
        const int b = bead[threadIdx.x];
        if (b >= 0) finish_bead<STEP>(s, b, s.mol_of[b], fsum[threadIdx.x], koff);
      }
      __syncthreads();
    }
  }
}

// The barrier alone, for the check that its wait ends: `rounds` barriers
// with `expected` arrivals (gridDim.x completes them; more makes every block
// wait out the limit).
__global__ void k_barrier_check(DevSys s, unsigned* bar, unsigned expected, int rounds,
                                unsigned long long limit_ns) {
  __shared__ unsigned gen0;
  if (threadIdx.x == 0) gen0 = ld_acquire_gpu(&bar[1]);
  __syncthreads();
  unsigned gen = gen0;
  for (int r = 0; r < rounds; ++r)
    if (!grid_barrier(bar, expected, gen, limit_ns, s.flags)) return;
}

// End of a block of `steps` steps: advance each running molecule's step
// count (clamped to its budget).  A neighbour-list overflow freezes
// everything until the host regrows the list and re-runs the block.
__global__ void k_advance(DevSys s, int steps) {
  pdl_wait();
  pdl_release();
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (*s.flags & FLAG_NL_OVERFLOW) return;
  if (m == 0) *s.sys_step += steps;  // the context's clock (blocks completed)
  if (m >= s.nmol) return;
  const MolConst mc = s.mol[m];
  if (!mc.active || s.mol_status[m] != 0) return;
  long long st = s.mol_step[m] + steps;
  if (mc.nsteps >= 0 && st > mc.nsteps) st = mc.nsteps;
  s.mol_step[m] = st;
}

// ---------------------------------------------------------------- energy
// Per-bead FP32 terms over the bead's full rows (each pair counted from both
// beads, so halved), reduced in FP64: e_bnd, e_ang_ss, e_vdw_att, e_vdw_rep
// (energy.cu:194-225, 278-307, 369-442).  Partial sums per block.
__global__ void __launch_bounds__(256) k_energy(DevSys s, int mol_start, int mol_n, int m,
                                                 double* __restrict__ part) {
  __shared__ double red[4][8];
  int i = mol_start + blockIdx.x * blockDim.x + threadIdx.x;
  float eb = 0.f, ea = 0.f, eat = 0.f, erp = 0.f;
  if (i < mol_start + mol_n) {
    const int cur = (int)(s.mol_step[m] & 1);
    const float4* X = s.x[cur];
    const float4 xi = X[i];
    const float boxl = s.boxl;
    const int2 br = s.bond_row[i];
    for (int e = 0; e < br.y; ++e) {
      const float4 xj = X[s.bond_j[br.x + e]];
      const float r0 = s.bond_r0[br.x + e];
      float lx, ly, lz;
      float dx = diff_exact(xj.x, xi.x, lx), dy = diff_exact(xj.y, xi.y, ly),
            dz = diff_exact(xj.z, xi.z, lz);
      min_image3(dx, dy, dz, boxl);
      float r = sqrtf(dx * dx + dy * dy + dz * dz);
      float dev = d2_minus_r02(dx, dy, dz, lx, ly, lz, r0) / (r + r0);
      eb += log1pf(-dev * dev / s.R0sq);
    }
    const int2 ar = s.ang_row[i];
    for (int e = 0; e < ar.y; ++e) {
      const float4 xj = X[s.ang_j[ar.x + e]];
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      min_image3(dx, dy, dz, boxl);
      float inv = 1.0f / (dx * dx + dy * dy + dz * dz);
      ea += s.e_ss * inv * inv * inv;
    }
    const int abase = s.nat_row[i].x, acnt = s.pl_att_cnt[i];
    for (int e = 0; e < acnt; ++e) {
      const float4 q = s.pl_att[abase + e];
      const float4 xj = X[__float_as_int(q.x)];
      float lx, ly, lz;
      float dx = diff_exact(xj.x, xi.x, lx), dy = diff_exact(xj.y, xi.y, ly),
            dz = diff_exact(xj.z, xi.z, lz);
      min_image3(dx, dy, dz, boxl);
      float d2 = dx * dx + dy * dy + dz * dz;
      float sr = q.y * q.y / d2;
      float s3 = sr * sr * sr;
      float sm1 = -d2_minus_r02(dx, dy, dz, lx, ly, lz, q.y) / d2;
      // eps_e (s^6 - 2 s^3) = eps_e (s^3 (s^3 - 1) - s^3)
      eat += q.w * (s3 * sm1 * (sr * sr + sr + 1.0f) - s3);
    }
    const long long rbase = (long long)i * s.nl_stride;
    const int rcnt = s.pl_cnt[i];
    const int ti = type_of(xi);
    const int jbase = s.mol[m].start;
    for (int e = 0; e < rcnt; ++e) {
      const float4 xj = X[jbase + (int)s.pl_j[rbase + e]];
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      min_image3(dx, dy, dz, boxl);
      float u = s.sig2[ti][type_of(xj)] / (dx * dx + dy * dy + dz * dz);
      float u3 = u * u * u;
      erp += s.rep6 ? s.eps_rep * u3 : s.eps_rep * u3 * (u3 + 1.0f);
    }
  }
  double v[4] = {0.5 * (double)eb, 0.5 * (double)ea, 0.5 * (double)eat, 0.5 * (double)erp};
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    double x = v[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[t][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double x = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x += red[threadIdx.x][k];
    part[4 * blockIdx.x + threadIdx.x] = x;
  }
}

// Final FP64 sum of the per-block partials, in block order.
__global__ void k_energy_final(const double* __restrict__ part, int nblocks, double k_bnd_R0sq_half,
                               double* __restrict__ out) {
  if (threadIdx.x >= 4) return;
  double x = 0.0;
  for (int b = 0; b < nblocks; ++b) x += part[4 * b + threadIdx.x];
  if (threadIdx.x == 0) x *= -k_bnd_R0sq_half;  // e_bnd = -(k R0^2 / 2) sum log(...)
  out[threadIdx.x] = x;
}

// ----------------------------------------------------------- observables
// Q over all native contacts (each counted from its lower bead), the
// first and second moments of the coordinates for Rg^2, and sum v^2, in FP64
// (sop.cu:528-611).  Partials per block: {contacts, sx, sy, sz, sxx, svv}.
__global__ void __launch_bounds__(256) k_observables(DevSys s, int mol_start, int mol_n, int m,
                                                      double* __restrict__ part) {
  __shared__ double red[6][8];
  int i = mol_start + blockIdx.x * blockDim.x + threadIdx.x;
  double v[6] = {0, 0, 0, 0, 0, 0};
  if (i < mol_start + mol_n) {
    const int cur = (int)(s.mol_step[m] & 1);
    const float4* X = s.x[cur];
    const float4 xi = X[i];
    const int2 nr = s.nat_row[i];
    int cnt = 0;
    for (int e = 0; e < nr.y; ++e) {
      int j = s.nat_j[nr.x + e];
      if (j < i) continue;
      const float4 xj = X[j];
      float dx = __fsub_rn(xi.x, xj.x), dy = __fsub_rn(xi.y, xj.y),
            dz = __fsub_rn(xi.z, xj.z);
      min_image3(dx, dy, dz, s.boxl);
      float d = sqrtf(d2_exact(dx, dy, dz));
      if (__fdiv_rn(d, s.nat_par[nr.x + e].x) < 1.25f) ++cnt;
    }
    const float4 vi = s.v[i];
    v[0] = cnt;
    v[1] = xi.x; v[2] = xi.y; v[3] = xi.z;
    v[4] = (double)xi.x * xi.x + (double)xi.y * xi.y + (double)xi.z * xi.z;
    v[5] = (double)vi.x * vi.x + (double)vi.y * vi.y + (double)vi.z * vi.z;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    double x = v[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[t][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double x = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x += red[threadIdx.x][k];
    part[6 * blockIdx.x + threadIdx.x] = x;
  }
}

__global__ void k_observables_final(const double* __restrict__ part, int nblocks, int n, int nnat,
                                    double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double t[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int k = 0; k < 6; ++k) t[k] += part[6 * b + k];
  const double inv = 1.0 / n;
  const double mx = t[1] * inv, my = t[2] * inv, mz = t[3] * inv;
  out[0] = nnat ? t[0] / nnat : 0.0;                           // Q
  out[1] = t[4] * inv - (mx * mx + my * my + mz * mz);         // rgsq = sum_{i<j} d^2 / N^2
  out[2] = t[5] / (3.0 * n);                                   // kinT
  out[3] = t[0];                                               // contct_nat
}

// Every bead's current unwrapped coordinates (each molecule at its own step
// parity) in bead-id order, for one device-to-host copy.
__global__ void k_gather_current(DevSys s, float* __restrict__ out, int* __restrict__ flag_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && flag_out) *flag_out = *s.flags;  // a frozen context's coordinates are stale
  if (i >= s.nbead) return;
  int m = s.mol_of[i];
  const float4 x = m < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : s.x[(int)(s.mol_step[m] & 1)][i];
  out[3 * (long long)i] = x.x;       // packed xyz: one contiguous copy to the host
  out[3 * (long long)i + 1] = x.y;
  out[3 * (long long)i + 2] = x.z;
}

// ----------------------------------------------------------- launchers
static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

template <int G, bool SPLIT, bool WIN>
static void launch_step_gsw(const DevSys& s, int koff, bool step, int wcap, cudaStream_t st) {
  const unsigned blocks = cdiv(s.nlive, kStepThreads / G);
  const int T = kStepThreads;
  const size_t sm = WIN ? (size_t)wcap * sizeof(float4) : 0;
  if (s.uniform_type) {
    if (step) launch_pdl_smem(k_step<G, true, true, SPLIT, WIN>, blocks, T, sm, st, s, koff, wcap);
    else launch_pdl_smem(k_step<G, false, true, SPLIT, WIN>, blocks, T, sm, st, s, koff, wcap);
  } else {
    if (step) launch_pdl_smem(k_step<G, true, false, SPLIT, WIN>, blocks, T, sm, st, s, koff, wcap);
    else launch_pdl_smem(k_step<G, false, false, SPLIT, WIN>, blocks, T, sm, st, s, koff, wcap);
  }
  if (SPLIT) {
    if (step) launch_pdl(k_finish<true>, cdiv(s.nlive, 256), 256, st, s, koff);
    else launch_pdl(k_finish<false>, cdiv(s.nlive, 256), 256, st, s, koff);
  }
}

template <int G>
static void launch_step_g(const DevSys& s, bool split, int koff, bool step, int wcap,
                          cudaStream_t st) {
  if (wcap > 0) {
    if (split) launch_step_gsw<G, true, true>(s, koff, step, wcap, st);
    else launch_step_gsw<G, false, true>(s, koff, step, wcap, st);
  } else {
    if (split) launch_step_gsw<G, true, false>(s, koff, step, 0, st);
    else launch_step_gsw<G, false, false>(s, koff, step, 0, st);
  }
}

// Lanes per bead G in {2, 4, 8, 16}; split: force kernel + finish kernel;
// wcap > 0: stage each block's molecules (up to wcap beads) in shared memory.
void launch_step(const DevSys& s, int G, bool split, int koff, bool step, int wcap,
                 cudaStream_t st) {
  switch (G) {
    case 2: launch_step_g<2>(s, split, koff, step, wcap, st); break;
    case 4: launch_step_g<4>(s, split, koff, step, wcap, st); break;
    case 16: launch_step_g<16>(s, split, koff, step, wcap, st); break;
    default: launch_step_g<8>(s, split, koff, step, wcap, st); break;
  }
}

// The tiled form: one launch over `ntiles` tiles, then k_finish when some
// tile uses the two-kernel form.
void launch_step_tiles(const DevSys& s, int koff, bool step, const int4* tiles, int ntiles,
                       bool any_split, cudaStream_t st) {
  if (ntiles <= 0) return;
  if (s.uniform_type) {
    if (step) launch_pdl(k_step_tiles<true, true>, (unsigned)ntiles, kStepThreads, st, s, koff, tiles);
    else launch_pdl(k_step_tiles<false, true>, (unsigned)ntiles, kStepThreads, st, s, koff, tiles);
  } else {
    if (step) launch_pdl(k_step_tiles<true, false>, (unsigned)ntiles, kStepThreads, st, s, koff, tiles);
    else launch_pdl(k_step_tiles<false, false>, (unsigned)ntiles, kStepThreads, st, s, koff, tiles);
  }
  if (any_split) {
    if (step) launch_pdl(k_finish<true>, cdiv(s.nlive, 256), 256, st, s, koff);
    else launch_pdl(k_finish<false>, cdiv(s.nlive, 256), 256, st, s, koff);
  }
}

// Cooperative launch: every block is resident at once (the barrier needs it).
template <typename... KArgs, typename... Args>
static cudaError_t launch_coop(void (*kernel)(KArgs...), unsigned grid, unsigned block,
                               cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Blocks of the persistent form (lanes G, step or force-only, one bead type
// or two) that are resident at once on this device, at most one per chunk.
template <int G, bool STEP, bool UNI>
static int persist_grid(int nchunks) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_step_persist<G, STEP, UNI>, kStepThreads,
                                                0);
  const int resident = std::max(1, per) * std::max(1, sms);
  return std::max(1, std::min(resident, nchunks));
}

template <int G, bool STEP, bool UNI>
static cudaError_t launch_persist_gsu(const DevSys& s, int koff0, int count, unsigned* bar,
                                      unsigned long long limit_ns, cudaStream_t st) {
  const unsigned grid = (unsigned)persist_grid<G, STEP, UNI>((int)cdiv(s.nlive, kStepThreads / G));
  return launch_coop(k_step_persist<G, STEP, UNI>, grid, kStepThreads, st, s, koff0, count, bar,
                     grid, limit_ns);
}

template <int G>
static cudaError_t launch_persist_g(const DevSys& s, int koff0, int count, bool step,
                                    unsigned* bar, unsigned long long limit_ns, cudaStream_t st) {
  if (s.uniform_type) {
    if (step) return launch_persist_gsu<G, true, true>(s, koff0, count, bar, limit_ns, st);
    return launch_persist_gsu<G, false, true>(s, koff0, count, bar, limit_ns, st);
  }
  if (step) return launch_persist_gsu<G, true, false>(s, koff0, count, bar, limit_ns, st);
  return launch_persist_gsu<G, false, false>(s, koff0, count, bar, limit_ns, st);
}

// Steps koff0 .. koff0 + count - 1 (no list rebuild among them) in one
// cooperative launch; bar: the context's two barrier words.
cudaError_t launch_step_persist(const DevSys& s, int G, int koff0, int count, bool step,
                                unsigned* bar, unsigned long long limit_ns, cudaStream_t st) {
  switch (G) {
    case 2: return launch_persist_g<2>(s, koff0, count, step, bar, limit_ns, st);
    case 4: return launch_persist_g<4>(s, koff0, count, step, bar, limit_ns, st);
    case 16: return launch_persist_g<16>(s, koff0, count, step, bar, limit_ns, st);
    default: return launch_persist_g<8>(s, koff0, count, step, bar, limit_ns, st);
  }
}

template <int G>
static cudaError_t launch_block_g(const DevSys& s, int koff0, int count, bool step, cudaStream_t st) {
  const unsigned B = kBlockFormThreads;
  if (s.uniform_type) {
    if (step) return launch_pdl(k_step_block<G, true, true>, 1, B, st, s, koff0, count);
    return launch_pdl(k_step_block<G, false, true>, 1, B, st, s, koff0, count);
  }
  if (step) return launch_pdl(k_step_block<G, true, false>, 1, B, st, s, koff0, count);
  return launch_pdl(k_step_block<G, false, false>, 1, B, st, s, koff0, count);
}

// Steps koff0 .. koff0 + count - 1 (no list rebuild among them) in one block.
cudaError_t launch_step_block(const DevSys& s, int G, int koff0, int count, bool step,
                              cudaStream_t st) {
  switch (G) {
    case 2: return launch_block_g<2>(s, koff0, count, step, st);
    case 4: return launch_block_g<4>(s, koff0, count, step, st);
    case 16: return launch_block_g<16>(s, koff0, count, step, st);
    default: return launch_block_g<8>(s, koff0, count, step, st);
  }
}

// `rounds` barriers over the persistent form's grid with `missing` arrivals
// that never come (0: the barriers complete).
cudaError_t launch_barrier_check(const DevSys& s, int G, unsigned* bar, int missing, int rounds,
                                 unsigned long long limit_ns, cudaStream_t st) {
  const int nchunks = (int)cdiv(s.nlive, kStepThreads / G);
  int grid = 1;
  switch (G) {
    case 2: grid = persist_grid<2, true, true>(nchunks); break;
    case 4: grid = persist_grid<4, true, true>(nchunks); break;
    case 16: grid = persist_grid<16, true, true>(nchunks); break;
    default: grid = persist_grid<8, true, true>(nchunks); break;
  }
  return launch_coop(k_barrier_check, (unsigned)grid, kStepThreads, st, s, bar,
                     (unsigned)grid + (unsigned)missing, rounds, limit_ns);
}

// Opts every windowed step kernel in to wcap beads of dynamic shared memory
// (above the 48 KB default a kernel must ask for it).
template <int G>
static cudaError_t allow_window_g(int wcap) {
  const int bytes = wcap * (int)sizeof(float4);
  cudaError_t e = cudaSuccess;
#define SOP_ALLOW(STEP, UNI, SPLIT)                                                           \
  if (e == cudaSuccess)                                                                       \
    e = cudaFuncSetAttribute(k_step<G, STEP, UNI, SPLIT, true>,                               \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  SOP_ALLOW(true, true, true) SOP_ALLOW(true, true, false) SOP_ALLOW(true, false, true)
  SOP_ALLOW(true, false, false) SOP_ALLOW(false, true, true) SOP_ALLOW(false, true, false)
  SOP_ALLOW(false, false, true) SOP_ALLOW(false, false, false)
#undef SOP_ALLOW
  return e;
}

cudaError_t allow_step_window(int wcap) {
  cudaError_t e = allow_window_g<2>(wcap);
  if (e == cudaSuccess) e = allow_window_g<4>(wcap);
  if (e == cudaSuccess) e = allow_window_g<8>(wcap);
  if (e == cudaSuccess) e = allow_window_g<16>(wcap);
  return e;
}

void launch_gather_current(const DevSys& s, float* out, int* flag_out, cudaStream_t st) {
  k_gather_current<<<cdiv(s.nbead, 256), 256, 0, st>>>(s, out, flag_out);
}

void launch_advance(const DevSys& s, int steps, cudaStream_t st) {
  launch_pdl(k_advance, cdiv(s.nmol, 256), 256, st, s, steps);
}

void launch_energy(const DevSys& s, int mol_start, int mol_n, int m, double* part, double* out,
                   double k_bnd_R0sq_half, cudaStream_t st) {
  int nb = (int)cdiv(mol_n, 256);
  k_energy<<<nb, 256, 0, st>>>(s, mol_start, mol_n, m, part);
  k_energy_final<<<1, 32, 0, st>>>(part, nb, k_bnd_R0sq_half, out);
}

void launch_observables(const DevSys& s, int mol_start, int mol_n, int m, int nnat, double* part,
                        double* out, cudaStream_t st) {
  int nb = (int)cdiv(mol_n, 256);
  k_observables<<<nb, 256, 0, st>>>(s, mol_start, mol_n, m, part);
  k_observables_final<<<1, 32, 0, st>>>(part, nb, mol_n, nnat, out);
}

}  // namespace sop
