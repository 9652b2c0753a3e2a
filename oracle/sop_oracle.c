/*
 * sop_oracle.c -- CPU restatement of the SOP reference algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only as the checker
 * or as the timed CPU baseline; the GPU engine never calls it.
 *
 * Parity status: the reference (samchogroup/SOP) ships no tests, fixtures or
 * golden vectors.  This restatement is pinned against the reference's own
 * host routines compiled from its sources (oracle/build_ref.sh -> oracle/_ref,
 * fixtures in tests/golden/): FP32 energies (energy.cu:194-225, 278-307,
 * 369-442), observables (sop.cu:528-611) and the file loader (io.cpp:112-259).
 * Forces and the integrator exist in the reference only as CUDA kernels; they
 * are restated here from energy.cu:228-584 and sop.cu:421-484 and pinned by the
 * energy/force consistency tests (finite differences of the pinned energies).
 *
 * Two arithmetic families:
 *   *_f64  FP64 physics from FP32 inputs: the parity oracle for forces,
 *          energies and single integrator steps.
 *   *_f32  the reference's FP32 arithmetic: list membership predicates (which
 *          must be bit-exact) and the serial CPU baseline.
 * Build with -ffp-contract=off so no multiply-add is fused on any host.
 *
 * Indices are 0-based throughout; the reference stores 1-based 14-bit indices
 * with a 2-bit type (global.h:51-67) and the loaders convert.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* params[] layout shared by every entry point */
enum {
  P_KBND = 0,   /* FENE spring constant k (param.cpp:14) */
  P_R0 = 1,     /* FENE R0 (param.cpp:15) */
  P_EPS_SS = 2, /* i,i+2 soft-sphere epsilon (param.cpp:37) */
  P_SIG_SS = 3, /* i,i+2 soft-sphere sigma (param.cpp:35) */
  P_EPS_REP = 4,/* non-native repulsion epsilon (energy.cu:15-19, global.cpp:69-73) */
  P_BOXL = 5,   /* periodic box length (param.cpp:97) */
  P_REP6 = 6,   /* 0: eps*(s^12/r^12 + s^6/r^6) as the reference; 1: eps*(s/r)^6 only */
  P_NPARAM = 7
};

/* sigma_rep[itype][jtype] (energy.cu:9-13, global.cpp:81-85); types are 1 or 2 */
static const double kSigmaRep[3][3] = {{0.0, 0.0, 0.0}, {0.0, 3.8, 5.4}, {0.0, 5.4, 7.0}};
static const float kSigmaRepF[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 3.8f, 5.4f}, {0.0f, 5.4f, 7.0f}};

static inline int tp(const int* type, int i) { return type ? type[i] : 1; }

/* ---------------------------------------------------------------- FP64 */

static inline double mi64(double d, double boxl) { return d - boxl * rint(d / boxl); }

static inline void delta64(const float* x, int i, int j, double boxl, double* d) {
  d[0] = mi64((double)x[3 * j + 0] - (double)x[3 * i + 0], boxl);
  d[1] = mi64((double)x[3 * j + 1] - (double)x[3 * i + 1], boxl);
  d[2] = mi64((double)x[3 * j + 2] - (double)x[3 * i + 2], boxl);
}

/*
 * Conservative forces and energy terms in FP64 on the given lists.
 *   bonds  (bi, bj, br0)           FENE          energy.cu:194-273
 *   angles (ai, ak)                i,i+2 soft sphere  energy.cu:278-362
 *   att    (pai, paj, pr0, peps)   native LJ 12-6     energy.cu:369-509
 *          peps_e: epsilon used by the energy (NULL: peps); the reference's
 *          energy uses coeff_att (global.cpp:51-55) which differs from the
 *          force's epsilon for type-(1,1) pairs.
 *   rep    (pri, prj)              non-native repulsion energy.cu:412-584
 * f: 3n doubles, overwritten.  e: 4 doubles (bnd, ang_ss, vdw_att, vdw_rep) or NULL.
 */
void orc_forces_f64(int n, const float* x, const int* type, int nbnd, const int* bi,
                    const int* bj, const float* br0, int nang, const int* ai, const int* ak,
                    int natt, const int* pai, const int* paj, const float* pr0,
                    const float* peps, const float* peps_e, long long nrep, const int* pri,
                    const int* prj, const double* params, double* f, double* e) {
  const double k = params[P_KBND], R0 = params[P_R0], R0sq = R0 * R0;
  const double eps_ss = params[P_EPS_SS], sig_ss = params[P_SIG_SS];
  const double eps_rep = params[P_EPS_REP], boxl = params[P_BOXL];
  const int rep6 = (int)params[P_REP6];
  const double sig_ss6 = pow(sig_ss, 6.0);
  double eb = 0.0, ea = 0.0, eat = 0.0, erp = 0.0;
  double d[3];
  memset(f, 0, sizeof(double) * 3 * (size_t)n);
  for (int b = 0; b < nbnd; ++b) {
    int i = bi[b], j = bj[b];
    delta64(x, i, j, boxl, d);
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double dev = r - (double)br0[b];
    double w = 1.0 - dev * dev / R0sq;
    eb += log(w);
    /* force on i: +k dev / (r w) * d  (energy.cu:255-271) */
    double c = k * dev / (r * w);
    for (int a = 0; a < 3; ++a) { f[3 * i + a] += c * d[a]; f[3 * j + a] -= c * d[a]; }
  }
  eb *= -k * R0sq / 2.0;
  for (int t = 0; t < nang; ++t) {
    int i = ai[t], j = ak[t];
    delta64(x, i, j, boxl, d);
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double r6 = r2 * r2 * r2;
    ea += eps_ss * sig_ss6 / r6;
    double c = 6.0 * eps_ss * sig_ss6 / (r6 * r2); /* energy.cu:344 */
    for (int a = 0; a < 3; ++a) { f[3 * i + a] -= c * d[a]; f[3 * j + a] += c * d[a]; }
  }
  for (int p = 0; p < natt; ++p) {
    int i = pai[p], j = paj[p];
    delta64(x, i, j, boxl, d);
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double s2 = (double)pr0[p] * (double)pr0[p] / r2;
    double s6 = s2 * s2 * s2, s12 = s6 * s6;
    double epsf = (double)peps[p];
    double epse = peps_e ? (double)peps_e[p] : epsf;
    eat += epse * (s12 - 2.0 * s6);
    double c = -12.0 * epsf / r2 * (s12 - s6); /* energy.cu:489-494 */
    for (int a = 0; a < 3; ++a) { f[3 * i + a] += c * d[a]; f[3 * j + a] -= c * d[a]; }
  }
  for (long long p = 0; p < nrep; ++p) {
    int i = pri[p], j = prj[p];
    delta64(x, i, j, boxl, d);
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double sg = kSigmaRep[tp(type, i)][tp(type, j)];
    double s2 = sg * sg / r2;
    double s6 = s2 * s2 * s2, s12 = s6 * s6;
    double c;
    if (rep6) {
      erp += eps_rep * s6;
      c = -6.0 * eps_rep / r2 * s6;
    } else {
      erp += eps_rep * (s12 + s6);
      c = -6.0 * eps_rep / r2 * (2.0 * s12 + s6); /* energy.cu:563-564 */
    }
    for (int a = 0; a < 3; ++a) { f[3 * i + a] += c * d[a]; f[3 * j + a] -= c * d[a]; }
  }
  if (e) { e[0] = eb; e[1] = ea; e[2] = eat; e[3] = erp; }
}

/* ------------------------------------------------------ Philox4x32-10 */
/* Counter-based RNG of Salmon, Moraes, Dror and Shaw (SC'11). */
void orc_philox4x32_10(const uint32_t* ctr_in, const uint32_t* key_in, uint32_t* out) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The engine's uniform: (float)r * 2^-32 + 2^-33, rounded in FP32, in (0, 1]. */
static inline float u01f(uint32_t r) {
  float rf = (float)r;
  float a = rf * 2.3283064365386963e-10f;
  return a + 1.1641532182693481e-10f;
}

/*
 * Standard normals of the engine's noise stream, in FP64 from the FP32
 * uniforms: counter (bead, step_lo, step_hi, traj), key (seed_lo, seed_hi);
 * Box-Muller on (u0, u1) gives x, y and on (u2, u3) gives z.
 * out: 3 * nbead doubles.
 */
void orc_noise_normals(int nbead, unsigned long long step, unsigned int traj,
                       unsigned long long seed, double* out) {
  const double two_pi = 6.283185307179586476925;
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int i = 0; i < nbead; ++i) {
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)step, (uint32_t)(step >> 32), traj};
    uint32_t r[4];
    orc_philox4x32_10(ctr, key, r);
    double u0 = u01f(r[0]), u1 = u01f(r[1]), u2 = u01f(r[2]), u3 = u01f(r[3]);
    double m0 = sqrt(-2.0 * log(u0)), m1 = sqrt(-2.0 * log(u2));
    out[3 * i + 0] = m0 * cos(two_pi * u1);
    out[3 * i + 1] = m0 * sin(two_pi * u1);
    out[3 * i + 2] = m1 * cos(two_pi * u3);
  }
}

/* ----------------------------------------------------- integrator, FP64 */
/*
 * Integrator constants of param.cpp:104-110 / 367-376 and the noise amplitude
 * of energy.cu:158.  out: a1, a2, a3, a4, sqrt(2 T zeta / h).
 */
void orc_langevin_consts(double h, double zeta, double T, double* out) {
  double halfh = h / 2.0;
  out[0] = h * (1.0 - zeta * halfh);
  out[1] = h * halfh;
  out[2] = (1.0 - h * zeta / 2.0 + (h * zeta) * (h * zeta) / 4.0) / h;
  out[3] = halfh * (1.0 - h * zeta / 2.0);
  out[4] = sqrt(2.0 * T * zeta / h);
}

/*
 * Position half of one underdamped step (sop.cu:421-447):
 *   incr = a1 v + a2 f; pos += incr (wrapped); unc_pos += incr.
 * All arrays 3n doubles, updated in place.
 */
void orc_position_update(int n, const double* c, double boxl, const double* v,
                         const double* f, double* incr, double* pos, double* unc) {
  for (int i = 0; i < 3 * n; ++i) {
    incr[i] = c[0] * v[i] + c[1] * f[i];
    double p = pos[i] + incr[i];
    pos[i] = p - boxl * rint(p / boxl);
    unc[i] += incr[i];
  }
}

/* Velocity half (sop.cu:450-462): v = a3 incr + a4 f. */
void orc_velocity_update(int n, const double* c, const double* incr, const double* f,
                         double* v) {
  for (int i = 0; i < 3 * n; ++i) v[i] = c[2] * incr[i] + c[3] * f[i];
}

/* ------------------------------------------------------- observables */
/*
 * Q (native contacts with d / r0 < 1.25 over all natives), Rg^2 as the
 * O(N^2) pair sum over N^2, and kinT = sum v^2 / (3N) (sop.cu:528-611), FP64.
 * out: Q, rgsq, kinT, contct_nat.
 */
void orc_observables(int n, const float* x, const float* v, int nnat, const int* ni,
                     const int* nj, const float* nr0, double boxl, double* out) {
  double d[3];
  long long cnt = 0;
  for (int c = 0; c < nnat; ++c) {
    delta64(x, nj[c], ni[c], boxl, d);
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (r / (double)nr0[c] < 1.25) ++cnt;
  }
  double rg = 0.0;
  for (int i = 0; i + 1 < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      delta64(x, j, i, boxl, d);
      rg += d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    }
  double sv = 0.0;
  if (v)
    for (int i = 0; i < 3 * n; ++i) sv += (double)v[i] * (double)v[i];
  out[0] = nnat ? (double)cnt / nnat : 0.0;
  out[1] = rg / ((double)n * (double)n);
  out[2] = sv / (3.0 * n);
  out[3] = (double)cnt;
}

/* ---------------------------------------------- lists, FP32 predicates */
/*
 * The list predicate of the reference's CPU filters (sop.cu:1370-1436,
 * 1737-1810): dx = x_j - x_i, minimum image, d2 = dx*dx + dy*dy + dz*dz in
 * FP32 left to right, member iff d2 < rcut2 (strict).  The minimum image is
 * applied only when |dx| > boxl/4; below that the reference's rounding term is
 * exactly zero, so the result is identical.
 */
static inline float mi32(float d, float boxl) {
  if (fabsf(d) > 0.25f * boxl) {
    float q = rintf(d / boxl);
    float s = boxl * q;
    d = d - s;
  }
  return d;
}

static inline float d2_32(const float* x, int i, int j, float boxl) {
  float dx = x[3 * j + 0] - x[3 * i + 0];
  float dy = x[3 * j + 1] - x[3 * i + 1];
  float dz = x[3 * j + 2] - x[3 * i + 2];
  dx = mi32(dx, boxl); dy = mi32(dy, boxl); dz = mi32(dz, boxl);
  float a = dx * dx;
  float b = dy * dy;
  float c = dz * dz;
  float s = a + b;
  return s + c;
}

/*
 * Squared cut-off as the reference forms it: rcut = fac * r in double rounded
 * to FP32 (sop.cu:746-747, 861-862), rcut2 = rcut * rcut in FP32.  A positive
 * fac selects the reference's factor mode; fac <= 0 selects an absolute
 * cut-off `absval` (A).
 */
float orc_rcut2(double fac, double absval, float r) {
  float rc = (fac > 0.0) ? (float)(fac * (double)r) : (float)absval;
  return rc * rc;
}

/*
 * Attractive list filter: keeps native entries c (indices into the native
 * arrays, or into `sel` when sel != NULL) with d2 < rcut2(fac, abs, r0).
 * Writes kept native indices to out, returns the count.
 */
int orc_filter_att(const float* x, int ncand, const int* sel, const int* ni, const int* nj,
                   const float* nr0, double fac, double absval, double boxl, int* out) {
  int k = 0;
  for (int t = 0; t < ncand; ++t) {
    int c = sel ? sel[t] : t;
    float rc2 = orc_rcut2(fac, absval, nr0[c]);
    if (d2_32(x, ni[c], nj[c], (float)boxl) < rc2) out[k++] = c;
  }
  return k;
}

/*
 * Repulsive neighbour list over the implicit master list: every pair i < j
 * with j - i > 2 that is not a native contact (the content of the
 * reference's idx_bead_lj_non_nat, io.cpp:216-225), filtered with
 * d2 < rcut2(fac * sigma_rep[ti][tj] or absval).  Natives must be sorted by
 * (ni, nj) with ni < nj.  Writes at most cap pairs; returns the full count.
 */
long long orc_nl_rep(int n, const float* x, const int* type, int nnat, const int* ni,
                     const int* nj, double fac, double absval, double boxl, long long cap,
                     int* oi, int* oj) {
  float rc2t[3][3];
  for (int a = 1; a < 3; ++a)
    for (int b = 1; b < 3; ++b) rc2t[a][b] = orc_rcut2(fac, absval, kSigmaRepF[a][b]);
  long long k = 0;
  int c = 0;
  for (int i = 0; i < n; ++i) {
    while (c < nnat && ni[c] < i) ++c;
    int cc = c;
    for (int j = i + 3; j < n; ++j) {
      while (cc < nnat && ni[cc] == i && nj[cc] < j) ++cc;
      if (cc < nnat && ni[cc] == i && nj[cc] == j) continue; /* native */
      if (d2_32(x, i, j, (float)boxl) < rc2t[tp(type, i)][tp(type, j)]) {
        if (k < cap) { oi[k] = i; oj[k] = j; }
        ++k;
      }
    }
  }
  return k;
}

/* Repulsive pair list: filter of an explicit pair list with the same predicate. */
long long orc_filter_rep(const float* x, const int* type, long long ncand, const int* ci,
                         const int* cj, double fac, double absval, double boxl, int* oi,
                         int* oj) {
  float rc2t[3][3];
  for (int a = 1; a < 3; ++a)
    for (int b = 1; b < 3; ++b) rc2t[a][b] = orc_rcut2(fac, absval, kSigmaRepF[a][b]);
  long long k = 0;
  for (long long p = 0; p < ncand; ++p) {
    int i = ci[p], j = cj[p];
    if (d2_32(x, i, j, (float)boxl) < rc2t[tp(type, i)][tp(type, j)]) {
      oi[k] = i; oj[k] = j; ++k;
    }
  }
  return k;
}

/* ------------------------------------------- serial FP32 CPU baseline */
/*
 * One molecule run with the reference's algorithm in FP32: the CPU
 * neighbour list over the O(N^2) master list every nnlup steps
 * (sop.cu:1354-1448), the CPU pair-list filter every nplup steps
 * (sop.cu:1710-1823), the four force kernels transcribed serially
 * (energy.cu:228-584), the noise force, and the two integrator kernels
 * (sop.cu:421-462).  Noise comes from the engine's Philox stream (the
 * reference's cuRAND XORWOW is a different generator; the cost of drawing
 * normals is comparable).  The list cut-offs are cut[0..3] = att_fac,
 * att_abs, rep_fac, rep_abs for the neighbour list and cut[4..7] for the
 * pair list.  The state persists between orc_ref_advance calls.
 */
typedef struct orc_ref {
  int n, nbnd, nang, nnat, nnlup, nplup;
  float *unc, *pos, *vel, *frc, *incr, *br0, *nr0, *neps;
  int *type, *bi, *bj, *ai, *ak, *ni, *nj;
  double params[P_NPARAM], cut[8];
  float a1, a2, a3, a4, var;
  int *nl_att, *pl_att, nnl_att, nil_att;
  int *nli, *nlj, *pli, *plj;
  long long nnl_rep, nil_rep, cap, step;
  uint32_t key[2];
  unsigned traj;
} orc_ref;

static void* dupmem(const void* src, size_t bytes) {
  void* p = malloc(bytes ? bytes : 1);
  if (p && src && bytes) memcpy(p, src, bytes);
  return p;
}

void orc_ref_destroy(orc_ref* r) {
  if (!r) return;
  free(r->unc); free(r->pos); free(r->vel); free(r->frc); free(r->incr);
  free(r->br0); free(r->nr0); free(r->neps); free(r->type); free(r->bi); free(r->bj);
  free(r->ai); free(r->ak); free(r->ni); free(r->nj); free(r->nl_att); free(r->pl_att);
  free(r->nli); free(r->nlj); free(r->pli); free(r->plj);
  free(r);
}

orc_ref* orc_ref_create(int n, const float* unc, const float* pos, const float* vel,
                        const int* type, int nbnd, const int* bi, const int* bj,
                        const float* br0, int nang, const int* ai, const int* ak, int nnat,
                        const int* ni, const int* nj, const float* nr0, const float* neps,
                        const double* params, const double* cut, double h, double zeta,
                        double T, int nnlup, int nplup, unsigned long long seed,
                        unsigned int traj) {
  orc_ref* r = (orc_ref*)calloc(1, sizeof(orc_ref));
  if (!r) return NULL;
  size_t f3 = sizeof(float) * 3 * (size_t)n;
  r->n = n; r->nbnd = nbnd; r->nang = nang; r->nnat = nnat; r->nnlup = nnlup; r->nplup = nplup;
  r->unc = (float*)dupmem(unc, f3);
  r->pos = (float*)dupmem(pos ? pos : unc, f3);
  r->vel = (float*)dupmem(vel, f3);
  if (!vel && r->vel) memset(r->vel, 0, f3);
  r->frc = (float*)calloc(3 * (size_t)n + 1, sizeof(float));
  r->incr = (float*)calloc(3 * (size_t)n + 1, sizeof(float));
  r->type = type ? (int*)dupmem(type, sizeof(int) * (size_t)n) : NULL;
  r->bi = (int*)dupmem(bi, sizeof(int) * (size_t)nbnd);
  r->bj = (int*)dupmem(bj, sizeof(int) * (size_t)nbnd);
  r->br0 = (float*)dupmem(br0, sizeof(float) * (size_t)nbnd);
  r->ai = (int*)dupmem(ai, sizeof(int) * (size_t)nang);
  r->ak = (int*)dupmem(ak, sizeof(int) * (size_t)nang);
  r->ni = (int*)dupmem(ni, sizeof(int) * (size_t)nnat);
  r->nj = (int*)dupmem(nj, sizeof(int) * (size_t)nnat);
  r->nr0 = (float*)dupmem(nr0, sizeof(float) * (size_t)nnat);
  r->neps = (float*)dupmem(neps, sizeof(float) * (size_t)nnat);
  memcpy(r->params, params, sizeof(r->params));
  memcpy(r->cut, cut, sizeof(r->cut));
  double cc[5];
  orc_langevin_consts(h, zeta, T, cc);
  r->a1 = (float)cc[0]; r->a2 = (float)cc[1]; r->a3 = (float)cc[2]; r->a4 = (float)cc[3];
  r->var = (float)cc[4];
  r->cap = (long long)n * 64 + 1024;
  r->nl_att = (int*)malloc(sizeof(int) * (size_t)(nnat + 1));
  r->pl_att = (int*)malloc(sizeof(int) * (size_t)(nnat + 1));
  r->nli = (int*)malloc(sizeof(int) * (size_t)r->cap);
  r->nlj = (int*)malloc(sizeof(int) * (size_t)r->cap);
  r->pli = (int*)malloc(sizeof(int) * (size_t)r->cap);
  r->plj = (int*)malloc(sizeof(int) * (size_t)r->cap);
  r->key[0] = (uint32_t)seed; r->key[1] = (uint32_t)(seed >> 32);
  r->traj = traj;
  r->step = -1;  /* step 0 (initial lists and forces) not yet done */
  if (!r->unc || !r->pos || !r->vel || !r->frc || !r->incr || !r->bi || !r->bj || !r->br0 ||
      !r->ai || !r->ak || !r->ni || !r->nj || !r->nr0 || !r->neps || !r->nl_att || !r->pl_att ||
      !r->nli || !r->nlj || !r->pli || !r->plj) {
    orc_ref_destroy(r);
    return NULL;
  }
  return r;
}

static int ref_lists(orc_ref* r, int nl, int pl) {
  const double boxl = r->params[P_BOXL];
  if (nl) {
    r->nnl_att = orc_filter_att(r->unc, r->nnat, NULL, r->ni, r->nj, r->nr0, r->cut[0], r->cut[1],
                                boxl, r->nl_att);
    for (;;) {
      long long need = orc_nl_rep(r->n, r->unc, r->type, r->nnat, r->ni, r->nj, r->cut[2],
                                  r->cut[3], boxl, r->cap, r->nli, r->nlj);
      if (need <= r->cap) { r->nnl_rep = need; break; }
      long long cap = need + need / 4;
      int* t[4];
      int** slot[4] = {&r->nli, &r->nlj, &r->pli, &r->plj};
      for (int q = 0; q < 4; ++q) {
        t[q] = (int*)realloc(*slot[q], sizeof(int) * (size_t)cap);
        if (!t[q]) return -1;
        *slot[q] = t[q];
      }
      r->cap = cap;
    }
  }
  if (pl) {
    r->nil_att = orc_filter_att(r->unc, r->nnl_att, r->nl_att, r->ni, r->nj, r->nr0, r->cut[4],
                                r->cut[5], boxl, r->pl_att);
    r->nil_rep = orc_filter_rep(r->unc, r->type, r->nnl_rep, r->nli, r->nlj, r->cut[6], r->cut[7],
                                boxl, r->pli, r->plj);
  }
  return 0;
}

/* force_eval: clear, noise, FENE, soft sphere, att, rep (energy.cu:81-150) */
static void ref_forces(orc_ref* r) {
  const int n = r->n;
  const float boxl = (float)r->params[P_BOXL];
  const float k_bnd = (float)r->params[P_KBND];
  const float R0sq = (float)(r->params[P_R0] * r->params[P_R0]);
  const float f_ang = (float)(6.0 * r->params[P_EPS_SS] * pow(r->params[P_SIG_SS], 6.0));
  const float eps_rep = (float)r->params[P_EPS_REP];
  float* unc = r->unc;
  float* frc = r->frc;
  memset(frc, 0, sizeof(float) * 3 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)r->step, (uint32_t)((unsigned long long)r->step >> 32),
                       r->traj};
    uint32_t q[4];
    orc_philox4x32_10(ctr, r->key, q);
    float m0 = sqrtf(-2.0f * logf(u01f(q[0])));
    float m1 = sqrtf(-2.0f * logf(u01f(q[2])));
    float t0 = 6.2831853f * u01f(q[1]), t1 = 6.2831853f * u01f(q[3]);
    frc[3 * i + 0] += r->var * m0 * cosf(t0);
    frc[3 * i + 1] += r->var * m0 * sinf(t0);
    frc[3 * i + 2] += r->var * m1 * cosf(t1);
  }
  for (int b = 0; b < r->nbnd; ++b) {
    int i = r->bi[b], j = r->bj[b];
    float dx = unc[3 * j] - unc[3 * i], dy = unc[3 * j + 1] - unc[3 * i + 1],
          dz = unc[3 * j + 2] - unc[3 * i + 2];
    dx -= boxl * rintf(dx / boxl); dy -= boxl * rintf(dy / boxl); dz -= boxl * rintf(dz / boxl);
    float d = sqrtf(dx * dx + dy * dy + dz * dz);
    float dev = d - r->br0[b];
    float tmp = -k_bnd * dev / d / (1.0f - dev * dev / R0sq);
    frc[3 * i] -= tmp * dx; frc[3 * i + 1] -= tmp * dy; frc[3 * i + 2] -= tmp * dz;
    frc[3 * j] += tmp * dx; frc[3 * j + 1] += tmp * dy; frc[3 * j + 2] += tmp * dz;
  }
  for (int t = 0; t < r->nang; ++t) {
    int i = r->ai[t], j = r->ak[t];
    float dx = unc[3 * j] - unc[3 * i], dy = unc[3 * j + 1] - unc[3 * i + 1],
          dz = unc[3 * j + 2] - unc[3 * i + 2];
    dx -= boxl * rintf(dx / boxl); dy -= boxl * rintf(dy / boxl); dz -= boxl * rintf(dz / boxl);
    float d = sqrtf(dx * dx + dy * dy + dz * dz);
    float co1 = f_ang / powf(d, 8.0f);
    frc[3 * i] -= co1 * dx; frc[3 * i + 1] -= co1 * dy; frc[3 * i + 2] -= co1 * dz;
    frc[3 * j] += co1 * dx; frc[3 * j + 1] += co1 * dy; frc[3 * j + 2] += co1 * dz;
  }
  for (int p = 0; p < r->nil_att; ++p) {
    int c = r->pl_att[p], i = r->ni[c], j = r->nj[c];
    float dx = unc[3 * j] - unc[3 * i], dy = unc[3 * j + 1] - unc[3 * i + 1],
          dz = unc[3 * j + 2] - unc[3 * i + 2];
    dx -= boxl * rintf(dx / boxl); dy -= boxl * rintf(dy / boxl); dz -= boxl * rintf(dz / boxl);
    float d2 = dx * dx + dy * dy + dz * dz;
    float r02 = r->nr0[c] * r->nr0[c];
    if (d2 > 1.0e-7f * r02) {
      float d6 = d2 * d2 * d2, d12 = d6 * d6;
      float r06 = r02 * r02 * r02, r012 = r06 * r06;
      float co1 = -12.0f * r->neps[c] / d2 * ((r012 / d12) - (r06 / d6));
      frc[3 * i] += co1 * dx; frc[3 * i + 1] += co1 * dy; frc[3 * i + 2] += co1 * dz;
      frc[3 * j] -= co1 * dx; frc[3 * j + 1] -= co1 * dy; frc[3 * j + 2] -= co1 * dz;
    }
  }
  for (long long p = 0; p < r->nil_rep; ++p) {
    int i = r->pli[p], j = r->plj[p];
    float dx = unc[3 * j] - unc[3 * i], dy = unc[3 * j + 1] - unc[3 * i + 1],
          dz = unc[3 * j + 2] - unc[3 * i + 2];
    dx -= boxl * rintf(dx / boxl); dy -= boxl * rintf(dy / boxl); dz -= boxl * rintf(dz / boxl);
    float sg = kSigmaRepF[tp(r->type, i)][tp(r->type, j)];
    float s2 = sg * sg, s6 = s2 * s2 * s2, s12 = s6 * s6;
    float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 > sg * 1.0e-7f) {
      float d6 = d2 * d2 * d2, d12 = d6 * d6;
      float co1 = -6.0f * eps_rep / d2 * (2.0f * s12 / d12 + s6 / d6);
      frc[3 * i] += co1 * dx; frc[3 * i + 1] += co1 * dy; frc[3 * i + 2] += co1 * dz;
      frc[3 * j] -= co1 * dx; frc[3 * j + 1] -= co1 * dy; frc[3 * j + 2] -= co1 * dz;
    }
  }
}

/* Advances nsteps steps (the first call also runs step 0, the initial lists
 * and forces of sop.cu:142-186).  Returns the steps run, or -1 on failure. */
long long orc_ref_advance(orc_ref* r, long long nsteps) {
  if (!r) return -1;
  const float boxl = (float)r->params[P_BOXL];
  const int n3 = 3 * r->n;
  if (r->step < 0) {
    r->step = 0;
    if (ref_lists(r, 1, 1)) return -1;
    ref_forces(r);
  }
  for (long long k = 0; k < nsteps; ++k) {
    const long long st = ++r->step;
    const int nl = r->nnlup > 0 && st % r->nnlup == 0;
    const int pl = nl || r->nplup <= 1 || st % r->nplup == 0;
    if ((nl || pl) && ref_lists(r, nl, pl)) return -1;
    for (int q = 0; q < n3; ++q) {
      r->incr[q] = r->a1 * r->vel[q] + r->a2 * r->frc[q];
      float p = r->pos[q] + r->incr[q];
      r->pos[q] = p - boxl * rintf(p / boxl);
      r->unc[q] += r->incr[q];
    }
    ref_forces(r);
    for (int q = 0; q < n3; ++q) r->vel[q] = r->a3 * r->incr[q] + r->a4 * r->frc[q];
  }
  return nsteps;
}

void orc_ref_state(const orc_ref* r, float* unc, float* pos, float* vel) {
  size_t f3 = sizeof(float) * 3 * (size_t)r->n;
  if (unc) memcpy(unc, r->unc, f3);
  if (pos) memcpy(pos, r->pos, f3);
  if (vel) memcpy(vel, r->vel, f3);
}

/* ------------------------------------------------------------------------
 * The reference's host Gaussian generator (random_generator.cpp:83-143): the
 * L'Ecuyer two-stream generator with a Bays-Durham shuffle ("ran2" of
 * Numerical Recipes, 2nd ed., section 7.1) and the polar Box-Muller method
 * ("gasdev", section 7.2), in the reference's types: FLOAT (float) results,
 * the constant expressions in double.  Seeded as `set run N` seeds it
 * (param.cpp:274-279: seed -100 - N).  With it the reference program built
 * without USE_CURAND draws var * gasdev() per bead and component, bead by
 * bead, x y z, at every force evaluation (energy.cu:168-188).
 */
typedef struct {
  int mseed, iset, idum2, iy, iv[32];
  float gset;
} orc_rangen;

static float rangen_ran2(orc_rangen* g) {
  const int IM1 = 2147483563, IM2 = 2147483399, IA1 = 40014, IA2 = 40692, IQ1 = 53668,
            IQ2 = 52774, IR1 = 12211, IR2 = 3791, NTAB = 32, IMM1 = IM1 - 1,
            NDIV = 1 + IMM1 / NTAB;
  const float AM = (float)(1.0 / (float)2147483563), RNMX = (float)(1.0 - 3.0e-16);
  int j, k;
  float temp;
  if (g->mseed <= 0) {
    g->mseed = (g->mseed == 0 ? 1 : -g->mseed);
    g->idum2 = g->mseed;
    for (j = NTAB + 7; j >= 0; j--) {
      k = g->mseed / IQ1;
      g->mseed = IA1 * (g->mseed - k * IQ1) - k * IR1;
      if (g->mseed < 0) g->mseed += IM1;
      if (j < NTAB) g->iv[j] = g->mseed;
    }
    g->iy = g->iv[0];
  }
  k = g->mseed / IQ1;
  g->mseed = IA1 * (g->mseed - k * IQ1) - k * IR1;
  if (g->mseed < 0) g->mseed += IM1;
  k = g->idum2 / IQ2;
  g->idum2 = IA2 * (g->idum2 - k * IQ2) - k * IR2;
  if (g->idum2 < 0) g->idum2 += IM2;
  j = g->iy / NDIV;
  g->iy = g->iv[j] - g->idum2;
  g->iv[j] = g->mseed;
  if (g->iy < 1) g->iy += IMM1;
  temp = AM * g->iy;
  return temp > RNMX ? RNMX : temp;
}

static float rangen_gasdev(orc_rangen* g) {
  float fac, rsq, v1, v2;
  if (g->iset == 0) {
    do {
      v1 = (float)(2.0 * rangen_ran2(g) - 1.0);
      v2 = (float)(2.0 * rangen_ran2(g) - 1.0);
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    /* the reference is C++ with `using namespace std`: log of a float is
       the float overload, the rest of the expression double */
    fac = (float)sqrt(-2.0 * logf(rsq) / rsq);
    g->gset = v1 * fac;
    g->iset = 1;
    return v2 * fac;
  }
  g->iset = 0;
  return g->gset;
}

/* `count` deviates of the generator after `set run` = run_id, from its
 * start (a fresh generator: iset 0, idum2 123456789, iy 0). */
void orc_ref_gasdev(int run_id, long long count, double* out) {
  orc_rangen g;
  memset(&g, 0, sizeof g);
  g.idum2 = 123456789;
  g.mseed = -100 - run_id;
  for (long long k = 0; k < count; ++k) out[k] = rangen_gasdev(&g);
}

/* ------------------------------------------------------------------------
 * Rg^2 as the reference computes it (calculate_observables, sop.cu:563-580):
 * every pair i < j in loop order, the minimum image with the host rnd()
 * (misc.cpp:4-11, half away from zero), and the sum of squared distances
 * accumulated in FLOAT (float), then divided by N^2.  For thousands of beads
 * the float sum of millions of positive terms loses low bits at every
 * addition, and the result falls below the exact value (-0.4% for 4,000
 * beads); this restatement reproduces that value bit for bit, so an engine
 * trajectory can be measured with the reference's own estimator.
 */
static float ref_rnd(float x) { return (float)((x > 0) ? floor(x + 0.5) : ceil(x - 0.5)); }

double orc_ref_rgsq(int n, const float* x, double boxl_d) {
  const float boxl = (float)boxl_d;
  float rg = 0.0f;
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j) {
      float dx = x[3 * i] - x[3 * j];
      float dy = x[3 * i + 1] - x[3 * j + 1];
      float dz = x[3 * i + 2] - x[3 * j + 2];
      dx -= boxl * ref_rnd(dx / boxl);
      dy -= boxl * ref_rnd(dy / boxl);
      dz -= boxl * ref_rnd(dz / boxl);
      rg += (dx * dx + dy * dy + dz * dz);
    }
  rg /= (float)(n * n);
  return rg;
}
