// Host side of libsopgpu.so: the context, device memory layout, the step
// loop captured as CUDA graphs, overflow recovery and the C ABI
// (include/sop_gpu.h).
//
// Replaces the reference's device-side host code: alloc_GPU_arrays /
// alloc_cudpp / setup_rng (GPUvars.cu:99-293, 417-453), force_eval /
// random_force (energy.cu:81-167), underdamped_iteration (sop.cu:466-484),
// update_neighbor_list / update_pair_list (sop.cu:928-1262, 1456-1706) and the
// per-step loop body of underdamped_ctrl (sop.cu:197-243).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "sop_dev.cuh"
#include "../../include/sop_gpu.h"

namespace sop {
// kernels_lists.cu
struct NLScratch {
  int* ncell;
  int* block_sums;
  int* cells_total;
};
void launch_nl_rebuild(const DevSys& s, const NLScratch& w, int koff, cudaStream_t st);
void launch_pl_rebuild(const DevSys& s, int koff, cudaStream_t st);
void launch_scan(const int* in, long long n, int* out, int* block_sums, cudaStream_t st);
long long scan_block_sums_needed(long long n);
// kernels_step.cu
void launch_step(const DevSys& s, int G, int koff, bool step, cudaStream_t st);
void launch_advance(const DevSys& s, int steps, cudaStream_t st);
void launch_gather_current(const DevSys& s, float4* out, cudaStream_t st);
void launch_energy(const DevSys& s, int mol_start, int mol_n, int m, double* part, double* out,
                   double k_bnd_R0sq_half, cudaStream_t st);
void launch_observables(const DevSys& s, int mol_start, int mol_n, int m, int nnat,
                        double* part, double* out, cudaStream_t st);
}  // namespace sop

using namespace sop;

namespace {

std::string g_lib_error;

struct HostMol {
  int n = 0;
  std::vector<int> bi, bj, ai, ak, ni, nj, types;
  std::vector<float> br0, nr0, neps, nepse, unc, pos, vel;
  double T = 0.6;
  unsigned traj = 0;
  long long nsteps = -1;
  int start = 0;
};

// sigma_rep[itype][jtype] (energy.cu:9-13)
const float kSigmaRep[3][3] = {{0.f, 0.f, 0.f}, {0.f, 3.8f, 5.4f}, {0.f, 5.4f, 7.0f}};

// The reference's cut-off: rcut = fac * r in double, rounded to FP32
// (sop.cu:746-747), or an absolute value; squared in FP32.
float rcut_of(double fac, double absval, float r) {
  return (fac > 0.0) ? (float)(fac * (double)r) : (float)absval;
}
float rcut2_of(double fac, double absval, float r) {
  float rc = rcut_of(fac, absval, r);
  return rc * rc;
}

float bits_f(int v) {
  float f;
  std::memcpy(&f, &v, sizeof f);
  return f;
}
int bits_i(float v) {
  int i;
  std::memcpy(&i, &v, sizeof i);
  return i;
}

struct Graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
};

}  // namespace

struct SopCtx {
  sop_params P{};
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<HostMol> mols;
  bool committed = false;

  DevSys s{};
  std::vector<void*> allocs;
  long long bytes = 0;
  NLScratch w{};
  int G = 8;
  double* e_part = nullptr;   // energy / observable partials
  double* e_out = nullptr;    // 8 doubles
  double* h_out = nullptr;    // pinned copy of e_out
  float4* stage = nullptr;    // gather buffer of sop_download_all
  std::map<int, float> tuning;  // step-kernel time (ms) per lanes-per-bead candidate
  long long host_step = 0;    // common step of plain / batched contexts
  long long target_step = 0;  // step every molecule should reach after the queued work
  std::map<std::string, Graph> graphs;
  std::vector<MolConst> mc;

  ~SopCtx() { release(); }

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  template <class T>
  T* dalloc(size_t count) {
    void* p = nullptr;
    size_t b = sizeof(T) * (count ? count : 1);
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    allocs.push_back(p);
    bytes += (long long)b;
    return (T*)p;
  }
  void dfree(void* p) {
    if (!p) return;
    auto it = std::find(allocs.begin(), allocs.end(), p);
    if (it != allocs.end()) allocs.erase(it);
    cudaFree(p);
  }
  void drop_graphs() {
    for (auto& kv : graphs) {
      if (kv.second.e) cudaGraphExecDestroy(kv.second.e);
      if (kv.second.g) cudaGraphDestroy(kv.second.g);
    }
    graphs.clear();
  }
  void release() {
    drop_graphs();
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (h_out) cudaFreeHost(h_out);
    h_out = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

static SopCtx* C(void* p) { return static_cast<SopCtx*>(p); }

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ctx->cuda_fail(e_, #call); \
  } while (0)

namespace {

int lanes_for(const SopCtx* ctx) {
  int g = ctx->P.lanes_per_bead;
  if (g == 2 || g == 4 || g == 8 || g == 16) return g;
  return 0;  // autotune
}

// Picks the lanes per bead G of the step kernel for this context by timing
// the force-only kernel (idempotent: it recomputes the same forces and
// look-ahead from the same state) for each G; results are bit-identical for
// every G, so only the speed differs.
int autotune_lanes(SopCtx* ctx) {
  const int cand[4] = {2, 4, 8, 16};
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  float best = 1e30f;
  int bestg = 8;
  for (int g : cand) {
    launch_step(ctx->s, g, 0, false, ctx->stream);  // warm-up
    CK(cudaEventRecord(a, ctx->stream));
    for (int r = 0; r < 3; ++r) launch_step(ctx->s, g, 0, false, ctx->stream);
    CK(cudaEventRecord(b, ctx->stream));
    CK(cudaEventSynchronize(b));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    ctx->tuning[g] = ms / 3.0f;
    if (ms < best) { best = ms; bestg = g; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->G = bestg;
  return SOP_OK;
}

// (Re)allocates the fixed-stride neighbour / pair-list rows.
int alloc_nl(SopCtx* ctx, long long stride) {
  stride = (stride + 31) / 32 * 32;  // rows stay 16-byte aligned
  const long long entries = stride * (long long)ctx->s.nbead;
  if (entries > 0x7fffffffLL) return ctx->fail(SOP_ERR_CAPACITY, "neighbour list exceeds 2^31 entries");
  ctx->dfree(ctx->s.nl_j);
  ctx->dfree(ctx->s.pl_j);
  ctx->s.nl_j = ctx->dalloc<int>(entries);
  ctx->s.pl_j = ctx->dalloc<int>(entries);
  if (!ctx->s.nl_j || !ctx->s.pl_j) return ctx->fail(SOP_ERR_ALLOC, "neighbour-list allocation failed");
  ctx->s.nl_stride = stride;
  ctx->drop_graphs();  // kernel arguments changed
  return SOP_OK;
}

// After a neighbour-list overflow: regrow the row stride to 1.25x the longest
// row the rebuild needed and clear the flag.  The stream must be idle.
int grow_nl(SopCtx* ctx) {
  int maxrow = 0;
  CK(cudaMemcpy(&maxrow, ctx->s.nl_maxrow, sizeof(int), cudaMemcpyDeviceToHost));
  long long stride = std::max<long long>(ctx->s.nl_stride + 32, (long long)maxrow * 5 / 4 + 32);
  int rc = alloc_nl(ctx, stride);
  if (rc) return rc;
  CK(cudaMemsetAsync(ctx->s.nl_maxrow, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->s.flags, 0, sizeof(int), ctx->stream));
  return SOP_OK;
}

// Neighbour-list rebuild that regrows the rows on overflow and rebuilds
// again.  Synchronous.
int nl_rebuild_checked(SopCtx* ctx, int koff) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    launch_nl_rebuild(ctx->s, ctx->w, koff, ctx->stream);
    CK(cudaGetLastError());
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!(flags & FLAG_NL_OVERFLOW)) return SOP_OK;
    int rc = grow_nl(ctx);
    if (rc) return rc;
  }
  return ctx->fail(SOP_ERR_CAPACITY, "neighbour list kept overflowing");
}

void force_eval_async(SopCtx* ctx) {
  launch_step(ctx->s, ctx->G, 0, false, ctx->stream);
}

// Which rebuilds precede step n (1-based): bit 0 neighbour list, bit 1 pair list.
int rebuilds_before(const sop_params& P, long long n) {
  int r = 0;
  if (P.nnlup > 0 && n % P.nnlup == 0) r |= 1;
  if ((r & 1) || P.nplup <= 1 || n % P.nplup == 0) r |= 2;
  return r;
}

// Launch sequence of steps s0+1 .. s0+count (koff 0 .. count-1) and the
// step-count advance.
void enqueue_block(SopCtx* ctx, long long s0, int count) {
  for (int k = 0; k < count; ++k) {
    int r = rebuilds_before(ctx->P, s0 + 1 + k);
    if (r & 1) launch_nl_rebuild(ctx->s, ctx->w, k, ctx->stream);
    if (r & 2) launch_pl_rebuild(ctx->s, k, ctx->stream);
    launch_step(ctx->s, ctx->G, k, true, ctx->stream);
  }
  launch_advance(ctx->s, count, ctx->stream);
}

int graph_for(SopCtx* ctx, long long s0, int count, cudaGraphExec_t* out) {
  std::string key(count, '0');
  for (int k = 0; k < count; ++k) key[k] = (char)('0' + rebuilds_before(ctx->P, s0 + 1 + k));
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    *out = it->second.e;
    return SOP_OK;
  }
  Graph g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_block(ctx, s0, count);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g.g);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&g.e, g.g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g.g);
    return ctx->cuda_fail(e, "cudaGraphInstantiate");
  }
  ctx->graphs[key] = g;
  *out = g.e;
  return SOP_OK;
}

int graph_steps(const SopCtx* ctx) {
  int P = ctx->P.graph_steps > 0 ? ctx->P.graph_steps : 10;
  return P;
}

// Queues nsteps steps of every molecule (no synchronisation).
int step_async(SopCtx* ctx, long long nsteps) {
  const int P = graph_steps(ctx);
  long long s0 = ctx->host_step;
  long long left = nsteps;
  while (left > 0) {
    long long phase = s0 % P;
    if (phase == 0 && left >= P) {
      cudaGraphExec_t ge;
      int rc = graph_for(ctx, s0, P, &ge);
      if (rc) return rc;
      CK(cudaGraphLaunch(ge, ctx->stream));
      s0 += P;
      left -= P;
    } else {
      int cnt = (int)std::min<long long>(left, P - phase);
      enqueue_block(ctx, s0, cnt);
      CK(cudaGetLastError());
      s0 += cnt;
      left -= cnt;
    }
  }
  ctx->host_step = s0;
  ctx->target_step = s0;
  return SOP_OK;
}

// Waits for queued work; on a neighbour-list overflow regrows the list and
// re-runs the steps that were skipped.
int sync_checked(SopCtx* ctx) {
  for (int round = 0; round < 8; ++round) {
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!(flags & FLAG_NL_OVERFLOW)) return SOP_OK;
    // Molecules froze at the start of the block that overflowed.  All of them
    // share one step (plain / batched contexts), read it from molecule 0.
    long long done = 0;
    int m0 = -1;
    for (size_t m = 0; m < ctx->mc.size(); ++m)
      if (ctx->mc[m].active) { m0 = (int)m; break; }
    if (m0 < 0) return SOP_OK;
    CK(cudaMemcpy(&done, ctx->s.mol_step + m0, sizeof(long long), cudaMemcpyDeviceToHost));
    int rc = grow_nl(ctx);
    if (rc) return rc;
    long long target = ctx->target_step;
    ctx->host_step = done;
    rc = step_async(ctx, target - done);
    if (rc) return rc;
  }
  return ctx->fail(SOP_ERR_CAPACITY, "neighbour list kept overflowing");
}

MolConst make_const(const sop_params& P, const HostMol& hm) {
  MolConst c{};
  c.start = hm.start;
  c.n = hm.n;
  double h = P.h, z = P.zeta, T = hm.T, halfh = h / 2.0;
  c.a1 = (float)(h * (1.0 - z * halfh));
  c.a2 = (float)(h * halfh);
  c.a3 = (float)((1.0 - h * z / 2.0 + (h * z) * (h * z) / 4.0) / h);
  c.a4 = (float)(halfh * (1.0 - h * z / 2.0));
  c.sigma_f = (float)std::sqrt(2.0 * T * z / h);
  c.t_zero = T < 1.0e-5 ? 1 : 0;
  c.traj = hm.traj;
  c.active = 1;
  c.nsteps = hm.nsteps;
  return c;
}

// Packs every staged molecule into the device layout.
int commit(SopCtx* ctx) {
  const sop_params& P = ctx->P;
  DevSys& s = ctx->s;
  int nbead = 0;
  for (auto& m : ctx->mols) {
    m.start = nbead;
    nbead += m.n;
  }
  const int nmol = (int)ctx->mols.size();
  if (nbead <= 0) return ctx->fail(SOP_ERR_ARG, "no beads");
  s.nbead = nbead;
  s.nmol = nmol;
  s.boxl = (float)P.boxl;
  s.eps_rep = (float)P.eps_rep;
  s.rep6 = P.rep6;
  s.k_bnd = (float)P.k_bnd;
  s.R0 = (float)P.R0;
  s.R0sq = (float)(P.R0 * P.R0);
  s.inv_R0sq = (float)(1.0 / (P.R0 * P.R0));
  double sig6 = std::pow(P.sigma_ss, 6.0);
  s.f_ss = (float)(6.0 * P.eps_ss * sig6);
  s.e_ss = (float)(P.eps_ss * sig6);
  float rcmax = 0.f;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      float sg = kSigmaRep[a][b];
      s.sig2[a][b] = sg * sg;
      s.rep_tol[a][b] = sg * 1.0e-7f;
      s.rc2_nl_rep[a][b] = rcut2_of(P.nl_rep_fac, P.nl_rep_abs, sg);
      s.rc2_pl_rep[a][b] = rcut2_of(P.pl_rep_fac, P.pl_rep_abs, sg);
      if (a > 0 && b > 0) rcmax = std::max(rcmax, rcut_of(P.nl_rep_fac, P.nl_rep_abs, sg));
    }
  s.rc_nl_rep_max = rcmax;
  s.seed_lo = (unsigned)(P.seed & 0xffffffffULL);
  s.seed_hi = (unsigned)(P.seed >> 32);

  // ---- host CSR rows (each pair in the rows of both beads)
  std::vector<int2> bond_row(nbead), ang_row(nbead), nat_row(nbead);
  std::vector<int> bond_j, ang_j, nat_j, mol_of(nbead);
  std::vector<float> bond_r0;
  std::vector<float4> nat_par;
  std::vector<float2> nat_rc2;
  std::vector<float4> x0(nbead), p0(nbead), v0(nbead);
  long long cell_cap = 0;
  {
    std::vector<int> cnt_b(nbead, 0), cnt_a(nbead, 0), cnt_n(nbead, 0);
    for (auto& m : ctx->mols) {
      for (size_t k = 0; k < m.bi.size(); ++k) { cnt_b[m.start + m.bi[k]]++; cnt_b[m.start + m.bj[k]]++; }
      for (size_t k = 0; k < m.ai.size(); ++k) { cnt_a[m.start + m.ai[k]]++; cnt_a[m.start + m.ak[k]]++; }
      for (size_t k = 0; k < m.ni.size(); ++k) { cnt_n[m.start + m.ni[k]]++; cnt_n[m.start + m.nj[k]]++; }
    }
    int ob = 0, oa = 0, on = 0;
    for (int i = 0; i < nbead; ++i) {
      bond_row[i] = make_int2(ob, 0); ob += cnt_b[i];
      ang_row[i] = make_int2(oa, 0); oa += cnt_a[i];
      nat_row[i] = make_int2(on, 0); on += cnt_n[i];
    }
    bond_j.resize(ob); bond_r0.resize(ob); ang_j.resize(oa);
    nat_j.resize(on); nat_par.resize(on); nat_rc2.resize(on);
    auto put_b = [&](int i, int j, float r0) {
      int e = bond_row[i].x + bond_row[i].y++;
      bond_j[e] = j; bond_r0[e] = r0;
    };
    auto put_a = [&](int i, int j) { ang_j[ang_row[i].x + ang_row[i].y++] = j; };
    auto put_n = [&](int i, int j, float r0, float ef, float ee) {
      int e = nat_row[i].x + nat_row[i].y++;
      nat_j[e] = j;
      nat_par[e] = make_float4(r0, ef, ee, 0.f);
      nat_rc2[e] = make_float2(rcut2_of(P.nl_att_fac, P.nl_att_abs, r0),
                               rcut2_of(P.pl_att_fac, P.pl_att_abs, r0));
    };
    for (int mi = 0; mi < nmol; ++mi) {
      auto& m = ctx->mols[mi];
      const int o = m.start;
      for (size_t k = 0; k < m.bi.size(); ++k) {
        put_b(o + m.bi[k], o + m.bj[k], m.br0[k]);
        put_b(o + m.bj[k], o + m.bi[k], m.br0[k]);
      }
      for (size_t k = 0; k < m.ai.size(); ++k) {
        put_a(o + m.ai[k], o + m.ak[k]);
        put_a(o + m.ak[k], o + m.ai[k]);
      }
      for (size_t k = 0; k < m.ni.size(); ++k) {
        put_n(o + m.ni[k], o + m.nj[k], m.nr0[k], m.neps[k], m.nepse[k]);
        put_n(o + m.nj[k], o + m.ni[k], m.nr0[k], m.neps[k], m.nepse[k]);
      }
      for (int i = 0; i < m.n; ++i) {
        mol_of[o + i] = mi;
        int t = m.types.empty() ? 1 : m.types[i];
        x0[o + i] = make_float4(m.unc[3 * i], m.unc[3 * i + 1], m.unc[3 * i + 2], bits_f(t));
        const std::vector<float>& pp = m.pos.empty() ? m.unc : m.pos;
        p0[o + i] = make_float4(pp[3 * i], pp[3 * i + 1], pp[3 * i + 2], 0.f);
        if (m.vel.empty()) v0[o + i] = make_float4(0.f, 0.f, 0.f, 0.f);
        else v0[o + i] = make_float4(m.vel[3 * i], m.vel[3 * i + 1], m.vel[3 * i + 2], 0.f);
      }
      cell_cap += std::max<long long>(64, 2LL * m.n);
    }
  }
  s.uniform_type = 1;
  for (auto& m : ctx->mols)
    for (int t : m.types)
      if (t != 1) s.uniform_type = 0;
  ctx->mc.resize(nmol);
  for (int mi = 0; mi < nmol; ++mi) ctx->mc[mi] = make_const(P, ctx->mols[mi]);

  // ---- device allocations
  const size_t nb = (size_t)nbead;
  for (int b = 0; b < 2; ++b) {
    s.x[b] = ctx->dalloc<float4>(nb);
    s.p[b] = ctx->dalloc<float4>(nb);
  }
  s.v = ctx->dalloc<float4>(nb);
  s.incr = ctx->dalloc<float4>(nb);
  s.f = ctx->dalloc<float4>(nb);
  s.mol_of = ctx->dalloc<int>(nb);
  MolConst* dmol = ctx->dalloc<MolConst>(nmol);
  s.mol = dmol;
  s.mol_step = ctx->dalloc<long long>(nmol);
  s.mol_status = ctx->dalloc<int>(nmol);
  s.bond_row = ctx->dalloc<int2>(nb);
  s.ang_row = ctx->dalloc<int2>(nb);
  s.nat_row = ctx->dalloc<int2>(nb);
  s.bond_j = ctx->dalloc<int>(bond_j.size());
  s.bond_r0 = ctx->dalloc<float>(bond_r0.size());
  s.ang_j = ctx->dalloc<int>(ang_j.size());
  s.nat_j = ctx->dalloc<int>(nat_j.size());
  s.nat_par = ctx->dalloc<float4>(nat_par.size());
  s.nat_rc2 = ctx->dalloc<float2>(nat_rc2.size());
  s.nl_att_cnt = ctx->dalloc<int>(nb);
  s.pl_att_cnt = ctx->dalloc<int>(nb);
  s.nl_att_e = ctx->dalloc<int>(nat_j.size());
  s.pl_att = ctx->dalloc<float4>(nat_j.size());
  s.nl_cnt = ctx->dalloc<int>(nb);
  s.pl_cnt = ctx->dalloc<int>(nb);
  s.nl_maxrow = ctx->dalloc<int>(1);
  s.nl_j = nullptr;
  s.pl_j = nullptr;
  {
    int rc = alloc_nl(ctx, 64);  // regrown from the first rebuild's longest row
    if (rc) return rc;
  }
  s.bbox = ctx->dalloc<unsigned>(6 * (size_t)nmol);
  s.grid = ctx->dalloc<MolGrid>(nmol);
  s.cell_cap = cell_cap;
  s.cell_cnt = ctx->dalloc<int>(cell_cap);
  s.cell_start = ctx->dalloc<int>(cell_cap + 1);
  s.bead_cell = ctx->dalloc<int>(nb);
  s.bead_slot = ctx->dalloc<int>(nb);
  s.sorted = ctx->dalloc<int>(nb);
  s.xs = ctx->dalloc<float4>(nb);
  s.flags = ctx->dalloc<int>(1);
  s.noise = nullptr;
  s.use_noise = 0;
  ctx->w.ncell = ctx->dalloc<int>(nmol);
  ctx->w.block_sums = ctx->dalloc<int>(scan_block_sums_needed(std::max<long long>(cell_cap, nbead)));
  ctx->w.cells_total = ctx->dalloc<int>(1);
  int maxn = 0;
  for (auto& m : ctx->mols) maxn = std::max(maxn, m.n);
  ctx->e_part = ctx->dalloc<double>(6 * ((size_t)maxn / 256 + 2));
  ctx->e_out = ctx->dalloc<double>(8);
  for (void* p : ctx->allocs)
    if (!p) return ctx->fail(SOP_ERR_ALLOC, "device allocation failed");
  if (!s.x[0] || !s.x[1] || !s.p[0] || !s.p[1] || !s.v || !s.incr || !s.f || !s.nl_j || !s.pl_j ||
      !s.cell_cnt || !s.cell_start || !ctx->e_part || !ctx->e_out || !ctx->w.block_sums)
    return ctx->fail(SOP_ERR_ALLOC, "device allocation failed");
  if (!ctx->h_out) CK(cudaMallocHost(&ctx->h_out, 8 * sizeof(double)));

  cudaStream_t st = ctx->stream;
  // x_0 sits in buffer 0 (step 0 is even)
  CK(cudaMemcpyAsync(s.x[0], x0.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.x[1], x0.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.p[0], p0.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.p[1], p0.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.v, v0.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(s.incr, 0, sizeof(float4) * nb, st));
  CK(cudaMemsetAsync(s.f, 0, sizeof(float4) * nb, st));
  CK(cudaMemcpyAsync(s.mol_of, mol_of.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dmol, ctx->mc.data(), sizeof(MolConst) * nmol, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(s.mol_step, 0, sizeof(long long) * nmol, st));
  CK(cudaMemsetAsync(s.mol_status, 0, sizeof(int) * nmol, st));
  CK(cudaMemcpyAsync(s.bond_row, bond_row.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.ang_row, ang_row.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(s.nat_row, nat_row.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, st));
  if (!bond_j.empty()) {
    CK(cudaMemcpyAsync(s.bond_j, bond_j.data(), sizeof(int) * bond_j.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s.bond_r0, bond_r0.data(), sizeof(float) * bond_r0.size(), cudaMemcpyHostToDevice, st));
  }
  if (!ang_j.empty())
    CK(cudaMemcpyAsync(s.ang_j, ang_j.data(), sizeof(int) * ang_j.size(), cudaMemcpyHostToDevice, st));
  if (!nat_j.empty()) {
    CK(cudaMemcpyAsync(s.nat_j, nat_j.data(), sizeof(int) * nat_j.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s.nat_par, nat_par.data(), sizeof(float4) * nat_par.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s.nat_rc2, nat_rc2.data(), sizeof(float2) * nat_rc2.size(), cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemsetAsync(s.flags, 0, sizeof(int), st));
  CK(cudaMemsetAsync(s.nl_att_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.pl_att_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.nl_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.pl_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.nl_maxrow, 0, sizeof(int), st));

  const int fixed_g = lanes_for(ctx);
  ctx->G = fixed_g ? fixed_g : 8;
  // set-up of underdamped_ctrl: lists from x_0, then f_0 and the look-ahead
  int rc = nl_rebuild_checked(ctx, 0);
  if (rc) return rc;
  launch_pl_rebuild(s, 0, st);
  force_eval_async(ctx);
  CK(cudaGetLastError());
  if (!fixed_g) {
    rc = autotune_lanes(ctx);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(st));
  ctx->host_step = 0;
  ctx->target_step = 0;
  ctx->committed = true;
  return SOP_OK;
}

int check_mol(SopCtx* ctx, int mol) {
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  if (mol < 0 || mol >= (int)ctx->mols.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown molecule");
  return SOP_OK;
}

int read_step(SopCtx* ctx, int mol, long long* step) {
  CK(cudaMemcpyAsync(ctx->h_out, ctx->s.mol_step + mol, sizeof(long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(step, ctx->h_out, sizeof(long long));
  return SOP_OK;
}

// float4 device rows -> 3 floats per bead on the host
int copy3(SopCtx* ctx, float* dst, const float4* src, int n) {
  CK(cudaMemcpy2DAsync(dst, 3 * sizeof(float), src, sizeof(float4), 3 * sizeof(float), n,
                       cudaMemcpyDeviceToHost, ctx->stream));
  return SOP_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

void sop_params_default(sop_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->k_bnd = 20.0;      // param.cpp:14
  p->R0 = 2.0;          // param.cpp:15
  p->eps_ss = 1.0;      // param.cpp:37
  p->sigma_ss = 3.5;    // param.cpp:35
  p->eps_rep = 1.0;     // energy.cu:15-19
  p->boxl = 500.0;      // param.cpp:97
  p->h = 2.5e-3;        // param.cpp:104
  p->zeta = 5.0e-2;     // param.cpp:100
  p->nl_att_fac = 3.2;  // sop.cu:746
  p->nl_rep_fac = 3.2;  // sop.cu:815
  p->pl_att_fac = 2.5;  // sop.cu:861
  p->pl_rep_fac = 2.5;  // sop.cu:910
  p->nnlup = 50;        // param.cpp:103
  p->nplup = 1;         // sop.cu:227-232: every step
  p->rep6 = 0;
  p->device = 0;
  p->graph_steps = 0;
  p->lanes_per_bead = 0;
  p->seed = 1234;       // setup_rng(1234, 0), sop.cu:138
}

int sop_ctx_create(const sop_params* p, void** out) {
  if (!p || !out) return SOP_ERR_ARG;
  *out = nullptr;
  if (p->boxl <= 0 || p->h <= 0 || p->R0 <= 0 || p->graph_steps < 0) {
    g_lib_error = "invalid parameters";
    return SOP_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(p->device);
  if (e != cudaSuccess) {
    g_lib_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  SopCtx* ctx = new SopCtx();
  ctx->P = *p;
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    g_lib_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    delete ctx;
    return SOP_ERR_CUDA;
  }
  *out = ctx;
  return SOP_OK;
}

int sop_ctx_destroy(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  cudaSetDevice(ctx->P.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return SOP_OK;
}

int sop_add_molecule(void* p, const sop_molecule* m, int* mol_id) {
  if (!p || !m) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->committed) return ctx->fail(SOP_ERR_ARG, "context already committed");
  if (m->nbead <= 0 || !m->unc_pos) return ctx->fail(SOP_ERR_ARG, "molecule needs beads and coordinates");
  if (m->nbnd < 0 || m->nang < 0 || m->nnat < 0) return ctx->fail(SOP_ERR_ARG, "negative counts");
  HostMol h;
  h.n = m->nbead;
  auto in = [&](int v) { return v >= 0 && v < m->nbead; };
  for (int k = 0; k < m->nbnd; ++k)
    if (!in(m->bond_i[k]) || !in(m->bond_j[k]) || m->bond_i[k] == m->bond_j[k])
      return ctx->fail(SOP_ERR_ARG, "bond index out of range");
  for (int k = 0; k < m->nang; ++k)
    if (!in(m->ang_i[k]) || !in(m->ang_k[k]) || m->ang_i[k] == m->ang_k[k])
      return ctx->fail(SOP_ERR_ARG, "angle index out of range");
  for (int k = 0; k < m->nnat; ++k)
    if (!in(m->nat_i[k]) || !in(m->nat_j[k]) || std::abs(m->nat_i[k] - m->nat_j[k]) <= 2)
      return ctx->fail(SOP_ERR_ARG, "native contact needs |i - j| > 2 and in-range indices");
  if (m->types)
    for (int i = 0; i < m->nbead; ++i)
      if (m->types[i] != 1 && m->types[i] != 2) return ctx->fail(SOP_ERR_ARG, "bead types must be 1 or 2");
  h.bi.assign(m->bond_i, m->bond_i + m->nbnd);
  h.bj.assign(m->bond_j, m->bond_j + m->nbnd);
  h.br0.assign(m->bond_r0, m->bond_r0 + m->nbnd);
  h.ai.assign(m->ang_i, m->ang_i + m->nang);
  h.ak.assign(m->ang_k, m->ang_k + m->nang);
  h.ni.assign(m->nat_i, m->nat_i + m->nnat);
  h.nj.assign(m->nat_j, m->nat_j + m->nnat);
  h.nr0.assign(m->nat_r0, m->nat_r0 + m->nnat);
  if (m->nat_eps) h.neps.assign(m->nat_eps, m->nat_eps + m->nnat);
  else h.neps.assign(m->nnat, 1.0f);
  if (m->nat_eps_energy) h.nepse.assign(m->nat_eps_energy, m->nat_eps_energy + m->nnat);
  else h.nepse = h.neps;
  if (m->types) h.types.assign(m->types, m->types + m->nbead);
  h.unc.assign(m->unc_pos, m->unc_pos + 3 * (size_t)m->nbead);
  if (m->pos) h.pos.assign(m->pos, m->pos + 3 * (size_t)m->nbead);
  if (m->vel) h.vel.assign(m->vel, m->vel + 3 * (size_t)m->nbead);
  h.T = m->T;
  h.traj = m->traj;
  h.nsteps = m->nsteps;
  ctx->mols.push_back(std::move(h));
  if (mol_id) *mol_id = (int)ctx->mols.size() - 1;
  return SOP_OK;
}

int sop_commit(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->committed) return ctx->fail(SOP_ERR_ARG, "context already committed");
  cudaSetDevice(ctx->P.device);
  return commit(ctx);
}

int sop_upload_topology(void* p, const sop_molecule* m) {
  int rc = sop_add_molecule(p, m, nullptr);
  if (rc) return rc;
  return sop_commit(p);
}

int sop_upload_state(void* p, int mol, const float* pos, const float* unc_pos, const float* vel) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long step;
  rc = read_step(ctx, mol, &step);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int cur = (int)(step & 1);
  std::vector<float4> buf(hm.n);
  std::vector<float4> old(hm.n);
  CK(cudaMemcpy(old.data(), ctx->s.x[cur] + hm.start, sizeof(float4) * hm.n, cudaMemcpyDeviceToHost));
  if (unc_pos) {
    for (int i = 0; i < hm.n; ++i)
      buf[i] = make_float4(unc_pos[3 * i], unc_pos[3 * i + 1], unc_pos[3 * i + 2], old[i].w);
    CK(cudaMemcpy(ctx->s.x[cur] + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  const float* pp = pos ? pos : unc_pos;
  if (pp) {
    for (int i = 0; i < hm.n; ++i) buf[i] = make_float4(pp[3 * i], pp[3 * i + 1], pp[3 * i + 2], 0.f);
    CK(cudaMemcpy(ctx->s.p[cur] + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  if (vel) {
    for (int i = 0; i < hm.n; ++i) buf[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f);
    CK(cudaMemcpy(ctx->s.v + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  rc = nl_rebuild_checked(ctx, 0);
  if (rc) return rc;
  launch_pl_rebuild(ctx->s, 0, ctx->stream);
  force_eval_async(ctx);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_step(void* p, long long nsteps) {
  if (!p || nsteps < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = step_async(ctx, nsteps);
  if (rc) return rc;
  return sync_checked(ctx);
}

int sop_step_async(void* p, long long nsteps) {
  if (!p || nsteps < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  return step_async(ctx, nsteps);
}

int sop_sync(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  return sync_checked(ctx);
}

int sop_launch_stage(void* p, int stage, int koff) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  switch (stage) {
    case 0: launch_step(ctx->s, ctx->G, koff, true, ctx->stream); break;
    case 1: launch_pl_rebuild(ctx->s, koff, ctx->stream); break;
    case 2: launch_nl_rebuild(ctx->s, ctx->w, koff, ctx->stream); break;
    case 3: launch_advance(ctx->s, koff, ctx->stream); break;
    default: return ctx->fail(SOP_ERR_ARG, "unknown stage");
  }
  CK(cudaGetLastError());
  return SOP_OK;
}

int sop_update_neighbor_list(void* p, long long* nnl_att, long long* nnl_rep) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  rc = nl_rebuild_checked(ctx, 0);
  if (rc) return rc;
  if (nnl_att || nnl_rep) {
    std::vector<int> a(ctx->s.nbead), r(ctx->s.nbead);
    CK(cudaMemcpy(a.data(), ctx->s.nl_att_cnt, sizeof(int) * a.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r.data(), ctx->s.nl_cnt, sizeof(int) * r.size(), cudaMemcpyDeviceToHost));
    long long sa = 0, sr = 0;
    for (int v : a) sa += v;
    for (int v : r) sr += v;
    if (nnl_att) *nnl_att = sa / 2;
    if (nnl_rep) *nnl_rep = sr / 2;
  }
  return SOP_OK;
}

int sop_update_pair_list(void* p, long long* nil_att, long long* nil_rep) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  launch_pl_rebuild(ctx->s, 0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (nil_att || nil_rep) {
    std::vector<int> a(ctx->s.nbead), r(ctx->s.nbead);
    CK(cudaMemcpy(a.data(), ctx->s.pl_att_cnt, sizeof(int) * a.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r.data(), ctx->s.pl_cnt, sizeof(int) * r.size(), cudaMemcpyDeviceToHost));
    long long sa = 0, sr = 0;
    for (int v : a) sa += v;
    for (int v : r) sr += v;
    if (nil_att) *nil_att = sa / 2;
    if (nil_rep) *nil_rep = sr / 2;
  }
  return SOP_OK;
}

int sop_force_eval(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  force_eval_async(ctx);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_set_noise(void* p, const float* normals) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  if (normals) {
    if (!ctx->s.noise) {
      ctx->s.noise = ctx->dalloc<float4>(ctx->s.nbead);
      if (!ctx->s.noise) return ctx->fail(SOP_ERR_ALLOC, "noise buffer allocation failed");
    }
    std::vector<float4> b(ctx->s.nbead);
    for (int i = 0; i < ctx->s.nbead; ++i)
      b[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.f);
    CK(cudaMemcpy(ctx->s.noise, b.data(), sizeof(float4) * b.size(), cudaMemcpyHostToDevice));
    ctx->s.use_noise = 1;
  } else {
    ctx->s.use_noise = 0;
  }
  ctx->drop_graphs();  // kernel arguments changed
  return SOP_OK;
}

int sop_download(void* p, int mol, float* pos, float* unc_pos, float* vel, float* force) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long step;
  rc = read_step(ctx, mol, &step);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int cur = (int)(step & 1);
  if (pos && (rc = copy3(ctx, pos, ctx->s.p[cur] + hm.start, hm.n))) return rc;
  if (unc_pos && (rc = copy3(ctx, unc_pos, ctx->s.x[cur] + hm.start, hm.n))) return rc;
  if (vel && (rc = copy3(ctx, vel, ctx->s.v + hm.start, hm.n))) return rc;
  if (force && (rc = copy3(ctx, force, ctx->s.f + hm.start, hm.n))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_download_list(void* p, int mol, int which, long long cap, int* i_out, int* j_out,
                      float* r0_out, long long* count) {
  if (!p || which < 0 || which > 3) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int n = hm.n, o = hm.start;
  long long k = 0;
  auto emit = [&](int i, int j, float r0) {
    if (j <= i) return;
    if (k < cap) {
      if (i_out) i_out[k] = i;
      if (j_out) j_out[k] = j;
      if (r0_out) r0_out[k] = r0;
    }
    ++k;
  };
  if (which == 0 || which == 2) {
    std::vector<int2> row(n);
    std::vector<int> cnt(n);
    CK(cudaMemcpy(row.data(), ctx->s.nat_row + o, sizeof(int2) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cnt.data(), (which == 0 ? ctx->s.nl_att_cnt : ctx->s.pl_att_cnt) + o,
                  sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (n > 0) {
      int lo = row[0].x, hi = row[n - 1].x + row[n - 1].y;
      size_t len = (size_t)std::max(hi - lo, 0);
      if (which == 0) {
        std::vector<int> e(len), nj(ctx->s.nbead > 0 ? len : 0);
        std::vector<float4> par(len);
        if (len) {
          CK(cudaMemcpy(e.data(), ctx->s.nl_att_e + lo, sizeof(int) * len, cudaMemcpyDeviceToHost));
          CK(cudaMemcpy(nj.data(), ctx->s.nat_j + lo, sizeof(int) * len, cudaMemcpyDeviceToHost));
          CK(cudaMemcpy(par.data(), ctx->s.nat_par + lo, sizeof(float4) * len, cudaMemcpyDeviceToHost));
        }
        for (int i = 0; i < n; ++i)
          for (int t = 0; t < cnt[i]; ++t) {
            int idx = e[row[i].x - lo + t] - lo;
            emit(i, nj[idx] - o, par[idx].x);
          }
      } else {
        std::vector<float4> q(len);
        if (len) CK(cudaMemcpy(q.data(), ctx->s.pl_att + lo, sizeof(float4) * len, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; ++i)
          for (int t = 0; t < cnt[i]; ++t) {
            float4 v = q[row[i].x - lo + t];
            emit(i, bits_i(v.x) - o, v.y);
          }
      }
    }
  } else {
    std::vector<int> cnt(n);
    CK(cudaMemcpy(cnt.data(), (which == 1 ? ctx->s.nl_cnt : ctx->s.pl_cnt) + o, sizeof(int) * n,
                  cudaMemcpyDeviceToHost));
    const long long stride = ctx->s.nl_stride;
    size_t len = (size_t)(stride * n);
    std::vector<int> jj(len);
    if (len)
      CK(cudaMemcpy(jj.data(), (which == 1 ? ctx->s.nl_j : ctx->s.pl_j) + stride * o,
                    sizeof(int) * len, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i)
      for (int t = 0; t < cnt[i]; ++t) emit(i, jj[(size_t)i * stride + t] - o, 0.f);
  }
  if (count) *count = k;
  return SOP_OK;
}

int sop_list_sizes(void* p, long long* out) {
  if (!p || !out) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  const int* src[4] = {ctx->s.nl_att_cnt, ctx->s.nl_cnt, ctx->s.pl_att_cnt, ctx->s.pl_cnt};
  std::vector<int> h(ctx->s.nbead);
  for (int t = 0; t < 4; ++t) {
    CK(cudaMemcpy(h.data(), src[t], sizeof(int) * h.size(), cudaMemcpyDeviceToHost));
    long long sum = 0;
    for (int v : h) sum += v;
    out[t] = sum / 2;  // full rows hold each pair twice
  }
  return SOP_OK;
}

int sop_download_all(void* p, float* unc_pos) {
  if (!p || !unc_pos) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  if (!ctx->stage) {
    ctx->stage = ctx->dalloc<float4>(ctx->s.nbead);
    if (!ctx->stage) return ctx->fail(SOP_ERR_ALLOC, "staging buffer allocation failed");
  }
  launch_gather_current(ctx->s, ctx->stage, ctx->stream);
  CK(cudaGetLastError());
  rc = copy3(ctx, unc_pos, ctx->stage, ctx->s.nbead);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_energy(void* p, int mol, double* terms) {
  if (!p || !terms) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  launch_energy(ctx->s, hm.start, hm.n, mol, ctx->e_part, ctx->e_out,
                0.5 * ctx->P.k_bnd * ctx->P.R0 * ctx->P.R0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_out, ctx->e_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; ++t) terms[t] = ctx->h_out[t];
  terms[4] = terms[0] + terms[1] + terms[2] + terms[3];  // rna_etot (energy.cu:76)
  return SOP_OK;
}

int sop_observables(void* p, int mol, double* out) {
  if (!p || !out) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  launch_observables(ctx->s, hm.start, hm.n, mol, (int)hm.ni.size(), ctx->e_part, ctx->e_out,
                     ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_out, ctx->e_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; ++t) out[t] = ctx->h_out[t];
  return SOP_OK;
}

int sop_molecule_status(void* p, int mol, int* status, long long* step) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long st = 0;
  int flags = 0;
  CK(cudaMemcpy(&st, ctx->s.mol_step + mol, sizeof(long long), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&flags, ctx->s.mol_status + mol, sizeof(int), cudaMemcpyDeviceToHost));
  const MolConst& mc = ctx->mc[mol];
  if (mc.nsteps >= 0 && st >= mc.nsteps) flags |= SOP_MOL_DONE;
  if (status) *status = flags;
  if (step) *step = st;
  return SOP_OK;
}

int sop_memory(void* p, int mol, long long* ctx_bytes, long long* mol_bytes) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx_bytes) *ctx_bytes = ctx->bytes;
  if (mol_bytes) {
    if (mol < 0 || mol >= (int)ctx->mols.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown molecule");
    const HostMol& hm = ctx->mols[mol];
    long long per_bead = 7 * 16 + 4 * 10 + 16 + 3 * 8;
    long long nl = ctx->s.nl_stride * 8LL * hm.n;
    *mol_bytes = per_bead * hm.n + nl + (long long)(hm.bi.size() + hm.ai.size()) * 16 +
                 (long long)hm.ni.size() * 2 * 40;
  }
  return SOP_OK;
}

int sop_tuning(void* p, int* lanes, float* ms) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (lanes) *lanes = ctx->G;
  if (ms) {
    const int cand[4] = {2, 4, 8, 16};
    for (int k = 0; k < 4; ++k) {
      auto it = ctx->tuning.find(cand[k]);
      ms[k] = it == ctx->tuning.end() ? 0.0f : it->second;
    }
  }
  return SOP_OK;
}

int sop_stream(void* p, void** stream) {
  if (!p || !stream) return SOP_ERR_ARG;
  *stream = (void*)C(p)->stream;
  return SOP_OK;
}

const char* sop_last_error(void* p) {
  if (!p) return g_lib_error.c_str();
  return C(p)->err.c_str();
}

}  // extern "C"
