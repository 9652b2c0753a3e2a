// Synthetic SOP native structures and the topology derived from them.
//
// The structures stand in for the PDB-derived input files the SOP program
// reads (bonds / angles / vdw / init, io.cpp:112-259).  A structure is a 3-D
// random walk with 3.8 A bonds, bond angles uniform in [80, 150] degrees,
// non-bonded beads at least 4.0 A apart (rejection sampling with
// back-tracking) and every bead inside a sphere of radius 3.8 * N^(1/3) * 1.2 A.
// From it come:
//   bonds    (i, i+1)    with r0 = native distance          (FENE, energy.cu:228-273)
//   angles   (i, i+1, i+2) with the native i..i+2 distance  (soft sphere, energy.cu:310-362)
//   natives  pairs |i-j| > 2 with native distance < 8.0 A   (LJ 12-6, energy.cu:445-509)
// Every other pair with |i-j| > 2 is a non-native (repulsive) pair, exactly
// the complement the reference's vdw file lists (io.cpp:203-225).
//
// Determinism: the walk uses its own xoshiro256** stream seeded through
// splitmix64 and its own series sin/cos/exp/log built from +,-,*,/ and sqrt
// only.  Compiled with -ffp-contract=off, an x86-64 and an aarch64 host give
// bit-identical structures for the same seed.
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <new>

namespace {

// ---------------------------------------------------------------- RNG
uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

struct Rng {  // xoshiro256** (Blackman & Vigna, 2018)
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) s[i] = splitmix64(x);
  }
  static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t result = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return result;
  }
  // uniform in [0, 1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ------------------------------------------------ deterministic elementary math
const double kPi = 3.14159265358979323846;
const double kTwoPi = 6.28318530717958647692;
const double kLn2 = 0.69314718055994530942;

// sin and cos of x by argument reduction to [-pi, pi] and Taylor series.
void det_sincos(double x, double* s, double* c) {
  double k = std::floor(x / kTwoPi + 0.5);
  double r = x - k * kTwoPi;
  double r2 = r * r;
  // sin r = r * sum_{n} (-1)^n r^{2n} / (2n+1)!, cos r = sum (-1)^n r^{2n}/(2n)!
  double ts = 1.0, tc = 1.0;  // Horner from the highest term (n = 14)
  for (int n = 14; n >= 1; --n) {
    ts = 1.0 - ts * r2 / ((2.0 * n) * (2.0 * n + 1.0));
    tc = 1.0 - tc * r2 / ((2.0 * n - 1.0) * (2.0 * n));
  }
  *s = r * ts;
  *c = tc;
}

double det_exp(double x) {
  double k = std::floor(x / kLn2 + 0.5);
  double r = x - k * kLn2;
  double t = 1.0;
  for (int n = 22; n >= 1; --n) t = 1.0 + t * r / n;
  return std::ldexp(t, (int)k);
}

double det_log(double x) {  // x > 0
  int e = 0;
  double m = std::frexp(x, &e);  // m in [0.5, 1)
  m *= 2.0; e -= 1;              // m in [1, 2)
  double t = (m - 1.0) / (m + 1.0);
  double t2 = t * t;
  double acc = 0.0;
  for (int n = 41; n >= 1; n -= 2) acc = 1.0 / n + acc * t2;
  return 2.0 * t * acc + e * kLn2;
}

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scl(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 unit(V3 a) { return scl(a, 1.0 / std::sqrt(dot(a, a))); }

const double kBond = 3.8;       // A
const double kExcl = 4.0;       // A, non-bonded minimum distance
const double kNatCut = 8.0;     // A, native-contact cut-off
const double kAngLo = 80.0 * kPi / 180.0;
const double kAngHi = 150.0 * kPi / 180.0;

// Uniform grid over [-R, R]^3 with per-cell LIFO chains; beads are removed
// in reverse order of insertion (back-tracking), so a removed bead is always
// the head of its cell.
struct Grid {
  double lo, cs;
  int nc;
  std::vector<int> head, next, cell_of;
  Grid(double R, double cell, int n) : lo(-R - cell), cs(cell) {
    nc = (int)std::ceil((2.0 * R + 2.0 * cell) / cell) + 1;
    head.assign((size_t)nc * nc * nc, -1);
    next.assign(n, -1);
    cell_of.assign(n, -1);
  }
  int coord(double v) const {
    int c = (int)std::floor((v - lo) / cs);
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
  }
  int cell(V3 p) const { return (coord(p.z) * nc + coord(p.y)) * nc + coord(p.x); }
  void insert(int i, V3 p) {
    int c = cell(p);
    next[i] = head[c]; head[c] = i; cell_of[i] = c;
  }
  void remove(int i) {
    int c = cell_of[i];
    head[c] = next[i];
    cell_of[i] = -1;
  }
};

}  // namespace

struct sopgen_mol {
  int n = 0;
  std::vector<float> xyz;  // 3n, float32-rounded native coordinates
  std::vector<int> nat_i, nat_j;
  std::vector<float> nat_r0, nat_eps;
};

static double dist_f(const float* a, const float* b) {
  double dx = (double)b[0] - (double)a[0];
  double dy = (double)b[1] - (double)a[1];
  double dz = (double)b[2] - (double)a[2];
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// Places n beads; returns 0 on success, 1 if the attempt budget ran out.
static int random_walk(int n, Rng& rng, std::vector<V3>& p) {
  const double R = kBond * std::cbrt((double)n) * 1.2;
  p.assign(n, V3{0, 0, 0});
  Grid grid(R, kExcl, n);
  p[0] = V3{0, 0, 0};
  grid.insert(0, p[0]);
  if (n == 1) return 0;
  int k = 1;
  int fails = 0;
  long long budget = 200000000LL;
  while (k < n) {
    bool placed = false;
    for (int attempt = 0; attempt < 64 && !placed; ++attempt) {
      if (--budget < 0) return 1;
      V3 w;
      if (k == 1) {
        double z = 2.0 * rng.uniform() - 1.0;
        double s, c;
        det_sincos(kTwoPi * rng.uniform(), &s, &c);
        double r = std::sqrt(1.0 - z * z);
        w = V3{r * c, r * s, z};
      } else {
        V3 u = unit(sub(p[k - 1], p[k - 2]));
        V3 a = std::fabs(u.x) < 0.9 ? V3{1, 0, 0} : V3{0, 1, 0};
        V3 e1 = unit(sub(a, scl(u, dot(a, u))));
        V3 e2 = cross(u, e1);
        double alpha = kAngLo + (kAngHi - kAngLo) * rng.uniform();
        double sa, ca, sp, cp;
        det_sincos(alpha, &sa, &ca);
        det_sincos(kTwoPi * rng.uniform(), &sp, &cp);
        // the bond angle at bead k-1 is the angle between -u and w
        w = add(scl(u, -ca), add(scl(e1, sa * cp), scl(e2, sa * sp)));
      }
      V3 q = add(p[k - 1], scl(w, kBond));
      if (dot(q, q) > R * R) continue;
      bool ok = true;
      int cx = grid.coord(q.x), cy = grid.coord(q.y), cz = grid.coord(q.z);
      for (int dz = -1; dz <= 1 && ok; ++dz)
        for (int dy = -1; dy <= 1 && ok; ++dy)
          for (int dx = -1; dx <= 1 && ok; ++dx) {
            int x = cx + dx, y = cy + dy, z = cz + dz;
            if (x < 0 || y < 0 || z < 0 || x >= grid.nc || y >= grid.nc || z >= grid.nc) continue;
            for (int j = grid.head[(z * grid.nc + y) * grid.nc + x]; j >= 0; j = grid.next[j]) {
              if (j == k - 1) continue;  // bonded neighbour
              V3 d = sub(q, p[j]);
              if (dot(d, d) < kExcl * kExcl) { ok = false; break; }
            }
          }
      if (!ok) continue;
      p[k] = q;
      grid.insert(k, q);
      ++k;
      placed = true;
    }
    if (placed) { fails = 0; continue; }
    // dead end: back-track further the longer we keep failing
    ++fails;
    int back = 1 << (fails < 6 ? fails : 6);
    if (back > k - 1) back = k - 1;
    for (int b = 0; b < back; ++b) { --k; grid.remove(k); }
    if (k < 1) k = 1;
  }
  return 0;
}

extern "C" {

// Generates the native structure and native contacts of an n-bead molecule.
// eps_lo == eps_hi gives every native contact that epsilon; otherwise each
// contact draws epsilon uniform in [eps_lo, eps_hi] from the same stream.
int sopgen_create(int n, uint64_t seed, double eps_lo, double eps_hi, sopgen_mol** out) {
  if (!out || n < 1) return 1;
  *out = nullptr;
  sopgen_mol* m = new (std::nothrow) sopgen_mol();
  if (!m) return 2;
  Rng rng(seed);
  std::vector<V3> p;
  if (random_walk(n, rng, p) != 0) { delete m; return 3; }
  m->n = n;
  m->xyz.resize(3 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    m->xyz[3 * i + 0] = (float)p[i].x;
    m->xyz[3 * i + 1] = (float)p[i].y;
    m->xyz[3 * i + 2] = (float)p[i].z;
  }
  // native contacts on the float32 coordinates, ordered by (i, j), i < j
  const double R = kBond * std::cbrt((double)n) * 1.2;
  Grid g(R + 1.0, kNatCut, n);
  std::vector<V3> pf(n);
  for (int i = 0; i < n; ++i)
    pf[i] = V3{(double)m->xyz[3 * i], (double)m->xyz[3 * i + 1], (double)m->xyz[3 * i + 2]};
  for (int i = 0; i < n; ++i) g.insert(i, pf[i]);
  std::vector<int> nb;
  for (int i = 0; i < n; ++i) {
    nb.clear();
    int cx = g.coord(pf[i].x), cy = g.coord(pf[i].y), cz = g.coord(pf[i].z);
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          int x = cx + dx, y = cy + dy, z = cz + dz;
          if (x < 0 || y < 0 || z < 0 || x >= g.nc || y >= g.nc || z >= g.nc) continue;
          for (int j = g.head[(z * g.nc + y) * g.nc + x]; j >= 0; j = g.next[j])
            if (j > i + 2) nb.push_back(j);
        }
    // insertion sort keeps the (i, j) order independent of the grid
    for (size_t a = 1; a < nb.size(); ++a) {
      int v = nb[a]; size_t b = a;
      while (b > 0 && nb[b - 1] > v) { nb[b] = nb[b - 1]; --b; }
      nb[b] = v;
    }
    for (int j : nb) {
      double d = dist_f(&m->xyz[3 * i], &m->xyz[3 * j]);
      if (d < kNatCut) {
        m->nat_i.push_back(i);
        m->nat_j.push_back(j);
        m->nat_r0.push_back((float)d);
      }
    }
  }
  m->nat_eps.resize(m->nat_i.size());
  for (size_t c = 0; c < m->nat_i.size(); ++c)
    m->nat_eps[c] = (eps_lo == eps_hi) ? (float)eps_lo
                                       : (float)(eps_lo + (eps_hi - eps_lo) * rng.uniform());
  *out = m;
  return 0;
}

void sopgen_destroy(sopgen_mol* m) { delete m; }

int sopgen_counts(const sopgen_mol* m, int* nbead, int* nbnd, int* nang, int* nnat) {
  if (!m) return 1;
  if (nbead) *nbead = m->n;
  if (nbnd) *nbnd = m->n > 1 ? m->n - 1 : 0;
  if (nang) *nang = m->n > 2 ? m->n - 2 : 0;
  if (nnat) *nnat = (int)m->nat_i.size();
  return 0;
}

int sopgen_native_xyz(const sopgen_mol* m, float* xyz) {
  if (!m || !xyz) return 1;
  std::memcpy(xyz, m->xyz.data(), sizeof(float) * 3 * (size_t)m->n);
  return 0;
}

// Bonds (i, i+1), 0-based, with the native bond length.
int sopgen_bonds(const sopgen_mol* m, int* bi, int* bj, float* r0) {
  if (!m) return 1;
  for (int i = 0; i + 1 < m->n; ++i) {
    bi[i] = i; bj[i] = i + 1;
    r0[i] = (float)dist_f(&m->xyz[3 * i], &m->xyz[3 * (i + 1)]);
  }
  return 0;
}

// Angles (i, i+1, i+2), 0-based, with the native i..i+2 distance.
int sopgen_angles(const sopgen_mol* m, int* ai, int* aj, int* ak, float* r_ik) {
  if (!m) return 1;
  for (int i = 0; i + 2 < m->n; ++i) {
    ai[i] = i; aj[i] = i + 1; ak[i] = i + 2;
    r_ik[i] = (float)dist_f(&m->xyz[3 * i], &m->xyz[3 * (i + 2)]);
  }
  return 0;
}

int sopgen_natives(const sopgen_mol* m, int* ni, int* nj, float* r0, float* eps) {
  if (!m) return 1;
  size_t c = m->nat_i.size();
  if (c) {
    std::memcpy(ni, m->nat_i.data(), sizeof(int) * c);
    std::memcpy(nj, m->nat_j.data(), sizeof(int) * c);
    std::memcpy(r0, m->nat_r0.data(), sizeof(float) * c);
    std::memcpy(eps, m->nat_eps.data(), sizeof(float) * c);
  }
  return 0;
}

// A fully extended chain: beads on the x axis, 3.8 A apart, centred on 0.
int sopgen_extended_xyz(int n, float* xyz) {
  if (n < 1 || !xyz) return 1;
  for (int i = 0; i < n; ++i) {
    xyz[3 * i + 0] = (float)((i - 0.5 * (n - 1)) * kBond);
    xyz[3 * i + 1] = 0.0f;
    xyz[3 * i + 2] = 0.0f;
  }
  return 0;
}

// Ensemble sizes and temperatures: n log-uniform in [n_lo, n_hi] (rounded to
// the nearest integer) and T uniform in [t_lo, t_hi].
int sopgen_ensemble(int count, int n_lo, int n_hi, double t_lo, double t_hi, uint64_t seed,
                    int* n_out, float* t_out) {
  if (count < 0 || n_lo < 1 || n_hi < n_lo) return 1;
  Rng rng(seed);
  double a = det_log((double)n_lo), b = det_log((double)n_hi);
  for (int i = 0; i < count; ++i) {
    double v = det_exp(a + (b - a) * rng.uniform());
    int n = (int)std::floor(v + 0.5);
    n_out[i] = n < n_lo ? n_lo : (n > n_hi ? n_hi : n);
    t_out[i] = (float)(t_lo + (t_hi - t_lo) * rng.uniform());
  }
  return 0;
}

// A served request stream: Poisson arrivals at `rate` per second for
// `duration` seconds.  Each job gets n log-uniform in [n_lo, n_hi], a step
// count log-uniform in [s_lo, s_hi], T uniform in [t_lo, t_hi]; even job ids
// start native, odd ones extended.  Returns the number of jobs written
// (at most `cap`) in *count.
int sopgen_requests(double rate, double duration, int n_lo, int n_hi, double s_lo, double s_hi,
                    double t_lo, double t_hi, uint64_t seed, int cap, int* count,
                    double* arrival, int* n_out, long long* steps_out, float* t_out,
                    int* extended_out) {
  if (rate <= 0 || duration < 0 || cap < 0 || !count) return 1;
  Rng rng(seed);
  double ln_lo = det_log((double)n_lo), ln_hi = det_log((double)n_hi);
  double ls_lo = det_log(s_lo), ls_hi = det_log(s_hi);
  double t = 0.0;
  int k = 0;
  while (k < cap) {
    double u = rng.uniform();
    t += -det_log(1.0 - u) / rate;
    if (t > duration) break;
    arrival[k] = t;
    double nv = det_exp(ln_lo + (ln_hi - ln_lo) * rng.uniform());
    int n = (int)std::floor(nv + 0.5);
    n_out[k] = n < n_lo ? n_lo : (n > n_hi ? n_hi : n);
    double sv = det_exp(ls_lo + (ls_hi - ls_lo) * rng.uniform());
    steps_out[k] = (long long)std::floor(sv + 0.5);
    t_out[k] = (float)(t_lo + (t_hi - t_lo) * rng.uniform());
    extended_out[k] = k & 1;
    ++k;
  }
  *count = k;
  return 0;
}

}  // extern "C"
