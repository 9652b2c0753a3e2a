// Device-side data layout and helpers of the SOP engine (sm_103a).
//
// Layout in HBM (one "system" = one or more independent molecules packed
// into one bead range; all arrays are structure-of-arrays):
//   x[2][nbead]   float4  unwrapped coordinates (unc_pos), ping-pong; w = bead
//                         type as int bits (1 or 2, the sigma_rep table index)
//   p[2][nbead]   float4  wrapped coordinates (pos), ping-pong
//   v, incr, f    float4  velocity, last position increment, force
//   mol_of        int     molecule slot of each bead (-1: free slot)
//   bond_row, ang_row, nat_row   int2 {start, count} into the topology pools;
//                         every bonded / angle / native pair is stored in the
//                         rows of both of its beads ("full" lists), so each
//                         bead sums its own force without atomics and the
//                         summation order is fixed
//   nl_j[nbead*stride] u16 repulsive neighbour list, fixed-stride rows: row i
//                         starts at i*nl_stride (64-byte aligned), holds
//                         nl_cnt[i] partners, each as its index minus the
//                         molecule's first bead (molecules hold at most
//                         65,535 beads); a row that would outgrow the stride
//                         raises the overflow flag and the host regrows
//   pl_cnt, pl_j    u16   repulsive pair list in the same row layout: row i
//                         is the first pl_cnt[i] entries at i*nl_stride (an
//                         in-order compaction of the neighbour-list row)
//   nl_att_cnt/nl_att_e   attractive neighbour list: native-entry indices in
//                         the native row layout
//   pl_att_cnt/pl_att     attractive pair list, float4 {j bits, r0, eps, 0}
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sop {

constexpr int kMaxLanes = 32;

// Per-molecule constants (written by the host at commit / admission).
struct MolConst {
  int start, n;                 // bead range
  float a1, a2, a3, a4;         // integrator constants (param.cpp:104-110)
  float sigma_f;                // sqrt(2 T zeta / h) (energy.cu:158)
  int t_zero;                   // T < 1e-5: no velocity update (sop.cu:479)
  unsigned traj;                // Philox stream id
  int active;                   // 1: stepping
  long long nsteps;             // step budget, < 0 unlimited
};

// Per-molecule cell grid of the neighbour-list build (device-computed).
struct MolGrid {
  float lo[3];
  float cs;                     // cell edge, A
  int dims[3];
  int S;                        // cells scanned on each side along each axis
  int base;                     // first global cell index
  int ncell;
  int brute;                    // 1: index-chunked cells, all pairs scanned
  int wrap;                     // 0: no pair of the molecule can reach boxl/4 (no minimum image)
};

struct DevSys {
  int nbead, nmol;
  int nlive;                    // bead slots the per-step kernels cover; every slot past it is free
  int only_mol;                 // >= 0: a list rebuild covers this molecule alone (a state upload)
  float boxl;
  float eps_rep;
  int rep6;
  float k_bnd, R0sq, R0, inv_R0sq;
  float f_ss;                   // 6 eps_ss sigma_ss^6 (param.cpp:36-39)
  float e_ss;                   // eps_ss sigma_ss^6
  float rc2_nl_rep[3][3];       // squared cut-offs by type pair
  float rc2_pl_rep[3][3];
  float rc_nl_rep_max;          // max neighbour-list cut-off (A)
  float sig2[3][3];             // sigma_rep^2 by type pair
  float rep_tol[3][3];          // sigma_rep * 1e-7: pairs with d^2 <= this are skipped (energy.cu:555-558)
  int uniform_type;             // 1: every bead has type 1 (one sigma for all pairs)
  int long_rows;                // 1: molecules of 10,000 beads or more (rows of ~400
                                // neighbours): the pair-list rebuild takes 16 lanes per bead
  unsigned seed_lo, seed_hi;

  float4* x[2];
  float4* p[2];
  float4* v;
  float4* incr;
  float4* f;
  float4* fsum;                 // conservative force of the step being taken; w: 0 idle,
                                // else marker bits (summed, a bond past R0, odd step)
  int* mol_of;
  const MolConst* mol;
  long long* mol_step;          // last completed step of each molecule (< 0: starts later)
  long long* sys_step;          // steps the context has completed (its clock)
  int* mol_status;              // SOP_MOL_* bits

  int2* bond_row; int* bond_j; float* bond_r0;
  int2* ang_row;  int* ang_j;
  int2* nat_row;  int* nat_j;  float4* nat_par;   // {r0, eps_f, eps_e, 0}
  float2* nat_rc2;              // {nl, pl} squared cut-offs per native entry

  int* nl_att_cnt; int* nl_att_e;
  int* pl_att_cnt; float4* pl_att;
  int* nl_cnt;
  unsigned short* nl_j;         // repulsive NL rows: partner - molecule start
  long long nl_stride;
  int* nl_maxrow;               // largest row a rebuild needed (for regrowth)
  int* pl_cnt;
  unsigned short* pl_j;         // repulsive PL rows, the same layout

  // neighbour-list build scratch
  unsigned* bbox;               // 6 per molecule, order-preserving float bits
  MolGrid* grid;
  int* cell_cnt; int* cell_start; long long cell_cap;
  int* bead_cell; int* bead_slot; int* sorted; float4* xs;
  int* flags;                   // bit 0: neighbour-list overflow
  float4* noise;                // injected normals or nullptr
  int use_noise;
};

enum { FLAG_NL_OVERFLOW = 1, FLAG_BARRIER_TIMEOUT = 2 };

// --------------------------------------------------------------- helpers
// Programmatic dependent launch.  The per-step kernels are launched with
// programmatic stream serialisation, so the next one's blocks may be
// scheduled while the previous kernel's last wave drains.  pdl_wait() blocks
// until the previous kernel on the stream has completed and its writes are
// visible (a no-op after an ordinary launch); pdl_release() lets the next
// kernel be scheduled.  Each such kernel waits before its first global access,
// so completion is transitive along the chain.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic stream serialisation (see pdl_wait).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block,
                              cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
// The same with dynamic shared memory.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_smem(void (*kernel)(KArgs...), unsigned grid, unsigned block,
                                   size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
__device__ __forceinline__ int type_of(float4 a) { return __float_as_int(a.w); }

// Entry (ti, tj) of a symmetric per-type-pair table (types are 1 or 2),
// selected in registers rather than indexed.
__device__ __forceinline__ float pick_type_pair(float a11, float a12, float a22, int ti, int tj) {
  return (ti == 1) ? (tj == 1 ? a11 : a12) : (tj == 1 ? a12 : a22);
}

// Minimum image exactly as the reference's filters produce it: the rounding
// term is zero whenever |d| <= boxl/4, so the division is skipped there.
__device__ __forceinline__ float min_image(float d, float boxl) {
  if (fabsf(d) > 0.25f * boxl) {
    float q = rintf(__fdiv_rn(d, boxl));
    d = __fsub_rn(d, __fmul_rn(boxl, q));
  }
  return d;
}

// Minimum image of a whole separation vector with one branch: the exact
// division runs only when some component exceeds boxl/4 (never for pairs on
// the lists of a molecule smaller than the box), so the common path is three
// compares.  Same results as min_image on each component.
__device__ __forceinline__ void min_image3(float& dx, float& dy, float& dz, float boxl) {
  if (fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz))) > 0.25f * boxl) {
    dx = min_image(dx, boxl);
    dy = min_image(dy, boxl);
    dz = min_image(dz, boxl);
  }
}

// FP32 squared distance formed left to right without fused multiply-adds,
// the arithmetic of the reference's host list filters (sop.cu:1378-1386):
// list membership decided on it is bit-exact with the oracle.
__device__ __forceinline__ float d2_exact(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Error-free transformations (Knuth two-sum, fma two-product).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// d^2 - r0^2 to a few ulps of the difference itself.  The separation is
// given as hi + lo per axis (the exact difference of the two FP32
// coordinates, see diff_exact); d^2 is formed in float-float and so is r0^2.
// This avoids the cancellation of (sqrt(d2) - r0) near the native distance,
// which would otherwise dominate the FENE and LJ force error: at the native
// structure those terms are ~1e-6 of the bead force while the FP32 rounding of
// x_j - x_i alone is ~1e-7 A.
__device__ __forceinline__ float d2_minus_r02(float dx, float dy, float dz, float lx, float ly,
                                              float lz, float r0) {
  float p0 = __fmul_rn(dx, dx), e0 = __fmaf_rn(dx, dx, -p0);
  float p1 = __fmul_rn(dy, dy), e1 = __fmaf_rn(dy, dy, -p1);
  float p2 = __fmul_rn(dz, dz), e2 = __fmaf_rn(dz, dz, -p2);
  float s01, t01;
  two_sum(p0, p1, s01, t01);
  float s, t;
  two_sum(s01, p2, s, t);
  float cross = __fmul_rn(2.0f, __fmaf_rn(dx, lx, __fmaf_rn(dy, ly, __fmul_rn(dz, lz))));
  float lo = __fadd_rn(__fadd_rn(__fadd_rn(t01, t), __fadd_rn(__fadd_rn(e0, e1), e2)), cross);
  float q = __fmul_rn(r0, r0), qe = __fmaf_rn(r0, r0, -q);
  float hi = __fsub_rn(s, q);   // exact when s and q are within a factor of 2
  return __fadd_rn(hi, __fsub_rn(lo, qe));
}

// a - b as hi + lo exactly (two-sum of a and -b); the caller minimum-images hi.
__device__ __forceinline__ float diff_exact(float a, float b, float& lo) {
  float hi;
  two_sum(a, -b, hi, lo);
  return hi;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Uniform in (0, 1]: (float)r * 2^-32 + 2^-33, each operation rounded.
__device__ __forceinline__ float u01(unsigned r) {
  return __fadd_rn(__fmul_rn(__uint2float_rn(r), 2.3283064365386963e-10f),
                   1.1641532182693481e-10f);
}

// Three standard normals for (bead, step) of trajectory traj: Box-Muller on
// (u0, u1) -> x, y and on (u2, u3) -> z.
__device__ __forceinline__ float3 noise3(unsigned bead, long long step, unsigned traj,
                                         unsigned seed_lo, unsigned seed_hi) {
  uint4 r = philox4x32_10(make_uint4(bead, (unsigned)step, (unsigned)((unsigned long long)step >> 32), traj),
                          make_uint2(seed_lo, seed_hi));
  float m0 = sqrtf(-2.0f * logf(u01(r.x)));
  float m1 = sqrtf(-2.0f * logf(u01(r.z)));
  float s0, c0, s1, c1;
  sincospif(2.0f * u01(r.y), &s0, &c0);
  sincospif(2.0f * u01(r.w), &s1, &c1);
  return make_float3(m0 * c0, m0 * s0, m1 * c1);
}

// Order-preserving float <-> uint for atomic min / max.
__device__ __forceinline__ unsigned f2ord(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

}  // namespace sop
