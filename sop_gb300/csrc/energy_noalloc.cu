// sop_energy_noalloc: the energy reduction for callers that may not
// allocate device memory.
//
// Who needs it: code that runs while device allocation is off limits -- a
// host application whose memory manager owns every device byte and hands out
// buffers itself, a loop that must not stall on the implicit device
// synchronisation cudaMalloc/cudaFree can bring, or an embedding where the
// surrounding framework forbids allocations outside its own pool.  Such a
// caller owns the input and output buffers; this entry point only launches
// kernels.
//
// It is a variant of the engine's energy reduction (k_energy + k_energy_final
// in kernels_step.cu), which keeps its per-block partial sums in scratch the
// context allocates.  Here the scratch is a file-scope __device__ array of
// fixed size (kMaxBlocks blocks of four doubles, 128 KiB) that every GPU
// loading this library holds until the process exits.  The lists are flat
// arrays of 0-based bead-index pairs with a separate per-bead type array,
// one thread per list entry, so no per-bead rows are needed.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <string>

#include "sop_dev.cuh"
#include "../../include/sop_gpu.h"

namespace sop {
namespace {

constexpr int kThreads = 256;
constexpr int kItemsPerThread = 4;
constexpr int kMaxBlocks = 4096;
constexpr long long kMaxItems = (long long)kMaxBlocks * kThreads * kItemsPerThread;

// Partial sums of the four energy terms, one group of four per block.  Each
// call writes the partials of every block it launches before the final sum
// reads them, so nothing has to start at zero; concurrent calls share it.
static __device__ __align__(256) double g_energy_scratch[kMaxBlocks * 4];

// Message of the calling thread's last failure.
thread_local std::string g_err;

struct Lists {
  int nbead;
  const float* x;
  const int* types;
  int nbnd; const int* bi; const int* bj; const float* br0;
  int nang; const int* ai; const int* ak;
  int natt; const int* pi; const int* pj; const float* pr0; const float* peps;
  long long nrep; const int* ri; const int* rj;
  float boxl, R0sq, e_ss, eps_rep;
  int rep6;
  float sig2[3][3];
};

__device__ __forceinline__ void separation(const float* x, int i, int j, float boxl, float& dx,
                                           float& dy, float& dz, float& lx, float& ly, float& lz) {
  dx = diff_exact(x[3 * j + 0], x[3 * i + 0], lx);
  dy = diff_exact(x[3 * j + 1], x[3 * i + 1], ly);
  dz = diff_exact(x[3 * j + 2], x[3 * i + 2], lz);
  min_image3(dx, dy, dz, boxl);
}

__device__ __forceinline__ bool bead_ok(int i, int nbead) { return i >= 0 && i < nbead; }

// One thread per list entry over [bonds | angles | native pairs | non-native
// pairs]; the same FP32 terms as k_energy, summed in FP64 per block.  An
// entry whose bead index lies outside [0, nbead), or whose bead type is not
// 1 or 2, is not evaluated: it adds NaN to its term, so the caller sees the
// bad input in that term and in rna_etot instead of an out-of-bounds read.
__global__ void __launch_bounds__(kThreads) k_energy_lists(Lists L, double* __restrict__ scratch) {
  __shared__ double red[4][kThreads / 32];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const double bad = __longlong_as_double(0x7ff8000000000000LL);  // quiet NaN
  const long long n1 = L.nbnd, n2 = n1 + L.nang, n3 = n2 + L.natt, n4 = n3 + L.nrep;
  const long long base = ((long long)blockIdx.x * kThreads + threadIdx.x) * kItemsPerThread;
  for (int q = 0; q < kItemsPerThread; ++q) {
    const long long e = base + q;
    if (e >= n4) break;
    float dx, dy, dz, lx, ly, lz;
    if (e < n1) {
      const int k = (int)e;
      if (!bead_ok(L.bi[k], L.nbead) || !bead_ok(L.bj[k], L.nbead)) { acc[0] += bad; continue; }
      separation(L.x, L.bi[k], L.bj[k], L.boxl, dx, dy, dz, lx, ly, lz);
      const float r0 = L.br0[k];
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      const float dev = d2_minus_r02(dx, dy, dz, lx, ly, lz, r0) / (r + r0);
      acc[0] += (double)log1pf(-dev * dev / L.R0sq);
    } else if (e < n2) {
      const int k = (int)(e - n1);
      if (!bead_ok(L.ai[k], L.nbead) || !bead_ok(L.ak[k], L.nbead)) { acc[1] += bad; continue; }
      separation(L.x, L.ai[k], L.ak[k], L.boxl, dx, dy, dz, lx, ly, lz);
      const float inv = 1.0f / (dx * dx + dy * dy + dz * dz);
      acc[1] += (double)(L.e_ss * inv * inv * inv);
    } else if (e < n3) {
      const int k = (int)(e - n2);
      if (!bead_ok(L.pi[k], L.nbead) || !bead_ok(L.pj[k], L.nbead)) { acc[2] += bad; continue; }
      separation(L.x, L.pi[k], L.pj[k], L.boxl, dx, dy, dz, lx, ly, lz);
      const float r0 = L.pr0[k];
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float sr = r0 * r0 / d2;
      const float s3 = sr * sr * sr;
      const float sm1 = -d2_minus_r02(dx, dy, dz, lx, ly, lz, r0) / d2;
      const float eps = L.peps ? L.peps[k] : 1.0f;
      acc[2] += (double)(eps * (s3 * sm1 * (sr * sr + sr + 1.0f) - s3));
    } else {
      const long long k = e - n3;
      const int i = L.ri[k], j = L.rj[k];
      if (!bead_ok(i, L.nbead) || !bead_ok(j, L.nbead)) { acc[3] += bad; continue; }
      const int ti = L.types ? L.types[i] : 1, tj = L.types ? L.types[j] : 1;
      if (ti < 1 || ti > 2 || tj < 1 || tj > 2) { acc[3] += bad; continue; }
      separation(L.x, i, j, L.boxl, dx, dy, dz, lx, ly, lz);
      const float u = pick_type_pair(L.sig2[1][1], L.sig2[1][2], L.sig2[2][2], ti, tj) /
                      (dx * dx + dy * dy + dz * dz);
      const float u3 = u * u * u;
      acc[3] += (double)(L.rep6 ? L.eps_rep * u3 : L.eps_rep * u3 * (u3 + 1.0f));
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    double v = acc[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[t][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int k = 0; k < kThreads / 32; ++k) v += red[threadIdx.x][k];
    scratch[4 * blockIdx.x + threadIdx.x] = v;
  }
}

// Final FP64 sum of the partials in block order (e_bnd gets -(k R0^2 / 2),
// energy.cu:223), then rna_etot (energy.cu:76).
__global__ void k_energy_lists_final(const double* __restrict__ scratch, int nblocks,
                                     double bnd_coeff, double* __restrict__ out) {
  __shared__ double t[4];
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int b = 0; b < nblocks; ++b) v += scratch[4 * b + threadIdx.x];
    if (threadIdx.x == 0) v *= -bnd_coeff;
    t[threadIdx.x] = v;
    out[threadIdx.x] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) out[4] = t[0] + t[1] + t[2] + t[3];
}

// Device address of the scratch array in the current device's current
// context.  The symbol's host-side name is not a device address, and the
// address belongs to a context (a context the caller made itself, or the
// primary context again after cudaDeviceReset, loads the array elsewhere), so
// it is looked up on every call rather than cached; the lookup is a host-side
// table read once the library's device code is loaded in that context.
cudaError_t scratch_for_current_context(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_energy_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

// sigma_rep[itype][jtype] (energy.cu:9-13)
const float kSig[3][3] = {{0.f, 0.f, 0.f}, {0.f, 3.8f, 5.4f}, {0.f, 5.4f, 7.0f}};

}  // namespace
}  // namespace sop

extern "C" {

int sop_energy_noalloc(const sop_params* p, const sop_energy_lists* l, double* terms,
                       void* stream) {
  using namespace sop;
  if (!p || !l || !terms || l->nbead <= 0 || !l->unc_pos || l->nbnd < 0 || l->nang < 0 ||
      l->natt < 0 || l->nrep < 0) {
    g_err = "sop_energy_noalloc: invalid arguments";
    return SOP_ERR_ARG;
  }
  if ((l->nbnd && (!l->bond_i || !l->bond_j || !l->bond_r0)) || (l->nang && (!l->ang_i || !l->ang_k)) ||
      (l->natt && (!l->att_i || !l->att_j || !l->att_r0)) || (l->nrep && (!l->rep_i || !l->rep_j))) {
    g_err = "sop_energy_noalloc: a non-empty list needs its index (and parameter) arrays";
    return SOP_ERR_ARG;
  }
  const long long items = (long long)l->nbnd + l->nang + l->natt + l->nrep;
  if (items > kMaxItems) {
    g_err = "sop_energy_noalloc: " + std::to_string(items) + " list entries exceed the maximum of " +
            std::to_string(kMaxItems) + " (the fixed scratch holds " + std::to_string(kMaxBlocks) +
            " block partials); use sop_energy on a context instead";
    return SOP_ERR_CAPACITY;
  }
  double* scratch = nullptr;
  cudaError_t e = scratch_for_current_context(&scratch);
  if (e != cudaSuccess) {
    g_err = std::string("sop_energy_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  Lists L;
  L.nbead = l->nbead; L.x = l->unc_pos; L.types = l->types;
  L.nbnd = l->nbnd; L.bi = l->bond_i; L.bj = l->bond_j; L.br0 = l->bond_r0;
  L.nang = l->nang; L.ai = l->ang_i; L.ak = l->ang_k;
  L.natt = l->natt; L.pi = l->att_i; L.pj = l->att_j; L.pr0 = l->att_r0; L.peps = l->att_eps;
  L.nrep = l->nrep; L.ri = l->rep_i; L.rj = l->rep_j;
  L.boxl = (float)p->boxl;
  L.R0sq = (float)(p->R0 * p->R0);
  L.e_ss = (float)(p->eps_ss * std::pow(p->sigma_ss, 6.0));
  L.eps_rep = (float)p->eps_rep;
  L.rep6 = p->rep6;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) L.sig2[a][b] = kSig[a][b] * kSig[a][b];
  const long long per_block = (long long)kThreads * kItemsPerThread;
  const int nb = (int)std::max<long long>(1, (items + per_block - 1) / per_block);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_energy_lists<<<nb, kThreads, 0, st>>>(L, scratch);
  k_energy_lists_final<<<1, 32, 0, st>>>(scratch, nb, 0.5 * p->k_bnd * p->R0 * p->R0, terms);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_err = std::string("sop_energy_noalloc: launch: ") + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  return SOP_OK;
}

const char* sop_energy_noalloc_error(void) { return sop::g_err.c_str(); }

}  // extern "C"
