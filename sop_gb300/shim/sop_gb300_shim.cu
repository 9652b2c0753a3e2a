// sop_gb300_shim.cu -- linked into a samchogroup/SOP build, it defines the
// reference's device-side entry points over the GB300 engine's C ABI
// (include/sop_gpu.h), so the reference's own parser, loaders, host energies,
// observables, output writers and step loop (underdamped_ctrl, sop.cu:104-285)
// run on this engine:
//   alloc_GPU_arrays   GPUvars.cu:99-231    -> sop_ctx_create + sop_upload_topology
//   alloc_cudpp        GPUvars.cu:232-298   -> nothing (the engine builds its lists)
//   setup_rng          GPUvars.cu:430-453   -> nothing (Philox keyed at creation)
//   update_neighbor_list / update_pair_list / update_cell_list /
//   update_hybrid_list sop.cu:928-2608      -> list sizes (rebuilt inside each step)
//   clear_forces, random_force energy.cu:54-67, 156-188 -> nothing
//   force_eval         energy.cu:81-150     -> sop_force_eval
//   underdamped_iteration sop.cu:466-484    -> sop_step(ctx, 1)
//
// The reference's loop reads its device arrays back every nup steps
// (sop.cu:252-263: dev_pos, dev_unc_pos, dev_vel, dev_idx_pair_list_att,
// dev_idx_pair_list_rep, dev_pl_lj_nat_pdb_dist) and then runs its host
// energy_eval and calculate_observables.  The shim keeps those six arrays as
// device mirrors and fills them from the engine after every nup-th step, so
// that block runs unchanged.
//
// Build (sop_gb300/shim/build_shim_ref.sh): the reference's objects with the
// definitions replaced here made weak (objcopy --weaken-symbol), this file,
// and sop_gb300/libsopgpu.so.  No reference source is edited.
//
// Check log: with SOP_SHIM_CHECK_FILE set, every mirror refresh appends one
// line of the engine's own energy terms and observables for the same state
// (step, e_bnd, e_ang_ss, e_vdw_rr_att, e_vdw_rr_rep, rna_etot, Q, rgsq,
// kinT, contct_nat) beside the reference's progress file.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "global.h"
#include "GPUvars.h"
#include "sop_gpu.h"

static void* g_ctx = nullptr;
static long long g_steps = 0;

static void sop_check(int rc, const char* what) {
  if (rc != SOP_OK) {  // the reference exits on any device failure
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, sop_last_error(g_ctx));
    exit(-1);
  }
}

static void cuda_check(cudaError_t rc, const char* what) {
  if (rc != cudaSuccess) {
    fprintf(stderr, "%s failed: %s\n", what, cudaGetErrorString(rc));
    exit(-1);
  }
}

static void publish_list_sizes() {
  long long s[4];
  sop_check(sop_list_sizes(g_ctx, s), "sop_list_sizes");
  nnl_att = (int)s[0]; nnl_rep = (int)s[1]; nil_att = (int)s[2]; nil_rep = (int)s[3];
}

static int type_of_bead(std::vector<int>& types) {
  types.assign(nbead, 1);
  for (int k = 0; k < ncon_att; ++k) {
    ushort2 c = idx_bead_lj_nat[k];
    types[GET_IDX(c.x) - 1] = GET_TYPE(c.x); types[GET_IDX(c.y) - 1] = GET_TYPE(c.y);
  }
  for (int k = 0; k < ncon_rep; ++k) {
    ushort2 c = idx_bead_lj_non_nat[k];
    types[GET_IDX(c.x) - 1] = GET_TYPE(c.x); types[GET_IDX(c.y) - 1] = GET_TYPE(c.y);
  }
  return 0;
}

// alloc_GPU_arrays (GPUvars.cu): builds the engine context from the globals
// the reference's loaders filled (io.cpp:112-259), 1-based 14-bit indices
// converted to 0-based.  A native contact's force epsilon is
// force_coeff_att[ti][tj] / -12 (the table of the force kernel,
// energy.cu:3-7) and its energy epsilon coeff_att[ti][tj] (the host energy,
// global.cpp:51-55, energy.cu:408-409), by the types of its two beads.
void alloc_GPU_arrays() {
  sop_params p;
  sop_params_default(&p);
  p.k_bnd = k_bnd; p.R0 = R0; p.eps_ss = epsilon_ss; p.sigma_ss = sigma_ss;
  p.eps_rep = coeff_rep[1][1]; p.boxl = boxl; p.h = h; p.zeta = zeta;
  p.nnlup = nnlup; p.nplup = 1;               // the reference's cadence
  p.device = deviceno;                        // set device (param.cpp:387-390)
  if (deviceno < 0) cuda_check(cudaGetDevice(&p.device), "cudaGetDevice");  // -1: the current one
  sop_check(sop_ctx_create(&p, &g_ctx), "sop_ctx_create");

  std::vector<int> bi(nbnd), bj(nbnd), ai(nang), ak(nang), ni(ncon_att), nj(ncon_att);
  std::vector<float> br0(nbnd), nr0(ncon_att), neps(ncon_att), neps_e(ncon_att);
  std::vector<float> x(3 * nbead), xp(3 * nbead), v(3 * nbead);
  std::vector<int> types;
  type_of_bead(types);
  for (int k = 0; k < nbnd; ++k) { bi[k] = ibead_bnd[k] - 1; bj[k] = jbead_bnd[k] - 1; br0[k] = pdb_dist[k]; }
  for (int k = 0; k < nang; ++k) { ai[k] = ibead_ang[k] - 1; ak[k] = kbead_ang[k] - 1; }
  for (int k = 0; k < ncon_att; ++k) {
    ushort2 c = idx_bead_lj_nat[k];
    const int ti = GET_TYPE(c.x), tj = GET_TYPE(c.y);
    ni[k] = GET_IDX(c.x) - 1; nj[k] = GET_IDX(c.y) - 1; nr0[k] = lj_nat_pdb_dist[k];
    neps[k] = (float)(force_coeff_att[ti][tj] / -12.0);
    neps_e[k] = (float)coeff_att[ti][tj];
  }
  for (int i = 0; i < nbead; ++i) {
    x[3 * i] = unc_pos[i].x; x[3 * i + 1] = unc_pos[i].y; x[3 * i + 2] = unc_pos[i].z;
    xp[3 * i] = pos[i].x;    xp[3 * i + 1] = pos[i].y;    xp[3 * i + 2] = pos[i].z;
    v[3 * i] = vel[i].x;     v[3 * i + 1] = vel[i].y;     v[3 * i + 2] = vel[i].z;
  }
  sop_molecule m = {};
  m.nbead = nbead;
  m.nbnd = nbnd; m.bond_i = bi.data(); m.bond_j = bj.data(); m.bond_r0 = br0.data();
  m.nang = nang; m.ang_i = ai.data(); m.ang_k = ak.data();
  m.nnat = ncon_att; m.nat_i = ni.data(); m.nat_j = nj.data(); m.nat_r0 = nr0.data();
  m.nat_eps = neps.data(); m.nat_eps_energy = neps_e.data();
  m.types = types.data(); m.unc_pos = x.data(); m.pos = xp.data(); m.vel = v.data();
  m.T = T; m.traj = 0; m.nsteps = -1;
  sop_check(sop_upload_topology(g_ctx, &m), "sop_upload_topology");
  publish_list_sizes();

  // device mirrors read by the loop's output block (sop.cu:252-263)
  pos_size = unc_pos_size = vel_size = nbead * sizeof(FLOAT3);
  cuda_check(cudaMalloc((void**)&dev_pos, pos_size), "cudaMalloc");
  cuda_check(cudaMalloc((void**)&dev_unc_pos, unc_pos_size), "cudaMalloc");
  cuda_check(cudaMalloc((void**)&dev_vel, vel_size), "cudaMalloc");
  cuda_check(cudaMalloc((void**)&dev_idx_pair_list_att, (ncon_att + 1) * sizeof(ushort2)), "cudaMalloc");
  cuda_check(cudaMalloc((void**)&dev_pl_lj_nat_pdb_dist, (ncon_att + 1) * sizeof(PDB_FLOAT)), "cudaMalloc");
  cuda_check(cudaMalloc((void**)&dev_idx_pair_list_rep, (ncon_rep + 1) * sizeof(ushort2)), "cudaMalloc");
}

void alloc_cudpp() {}                         // lists are built by the engine
void setup_rng(unsigned long long seed, unsigned long long offset) {
  (void)seed; (void)offset;                   // Philox keyed at context creation
}

// The engine rebuilds both lists on the cadence given at creation, inside
// each step; these publish the counts the host loop prints and reads.
void update_neighbor_list() { publish_list_sizes(); }
void update_pair_list() { publish_list_sizes(); }
void update_cell_list() { publish_list_sizes(); }
void update_hybrid_list() { publish_list_sizes(); }

void clear_forces() {}                        // forces are written, not accumulated
void force_eval() { sop_check(sop_force_eval(g_ctx), "sop_force_eval"); }
void random_force() {}                        // noise is part of every force evaluation

// The engine's state into the reference's host arrays: coordinates,
// velocities and the current pair lists (1-based, typed ushort2 records).
void sop_shim_fetch_for_output() {
  std::vector<float> xp(3 * nbead), xu(3 * nbead), v(3 * nbead);
  sop_check(sop_download(g_ctx, 0, xp.data(), xu.data(), v.data(), nullptr), "sop_download");
  for (int i = 0; i < nbead; ++i) {
    pos[i].x = xp[3 * i]; pos[i].y = xp[3 * i + 1]; pos[i].z = xp[3 * i + 2];
    unc_pos[i].x = xu[3 * i]; unc_pos[i].y = xu[3 * i + 1]; unc_pos[i].z = xu[3 * i + 2];
    vel[i].x = v[3 * i]; vel[i].y = v[3 * i + 1]; vel[i].z = v[3 * i + 2];
  }
  std::vector<int> type_of;
  type_of_bead(type_of);
  for (int which = 2; which <= 3; ++which) {
    long long n = 0;
    sop_check(sop_download_list(g_ctx, 0, which, 0, nullptr, nullptr, nullptr, &n), "sop_download_list");
    std::vector<int> i(n > 0 ? n : 1), j(n > 0 ? n : 1);
    std::vector<float> r0(n > 0 ? n : 1);
    sop_check(sop_download_list(g_ctx, 0, which, n, i.data(), j.data(), r0.data(), &n), "sop_download_list");
    ushort2* out = which == 2 ? idx_pair_list_att : idx_pair_list_rep;
    for (long long k = 0; k < n; ++k) {
      out[k].x = COMBINE(type_of[i[k]], i[k] + 1);
      out[k].y = COMBINE(type_of[j[k]], j[k] + 1);
      if (which == 2) pl_lj_nat_pdb_dist[k] = r0[k];
    }
    if (which == 2) nil_att = (int)n; else nil_rep = (int)n;
  }
}

// Fills the device mirrors from the engine, and appends the engine's own
// energy and observables to the check log when one is asked for.
static void refresh_mirrors() {
  sop_shim_fetch_for_output();
  cuda_check(cudaMemcpy(dev_pos, pos, pos_size, cudaMemcpyHostToDevice), "cudaMemcpy");
  cuda_check(cudaMemcpy(dev_unc_pos, unc_pos, unc_pos_size, cudaMemcpyHostToDevice), "cudaMemcpy");
  cuda_check(cudaMemcpy(dev_vel, vel, vel_size, cudaMemcpyHostToDevice), "cudaMemcpy");
  cuda_check(cudaMemcpy(dev_idx_pair_list_att, idx_pair_list_att, nil_att * sizeof(ushort2),
                        cudaMemcpyHostToDevice), "cudaMemcpy");
  cuda_check(cudaMemcpy(dev_pl_lj_nat_pdb_dist, pl_lj_nat_pdb_dist, nil_att * sizeof(PDB_FLOAT),
                        cudaMemcpyHostToDevice), "cudaMemcpy");
  cuda_check(cudaMemcpy(dev_idx_pair_list_rep, idx_pair_list_rep, nil_rep * sizeof(ushort2),
                        cudaMemcpyHostToDevice), "cudaMemcpy");
  const char* path = getenv("SOP_SHIM_CHECK_FILE");
  if (path && *path) {
    double e[5], ob[4];
    sop_check(sop_energy(g_ctx, 0, e), "sop_energy");
    sop_check(sop_observables(g_ctx, 0, ob), "sop_observables");
    FILE* f = fopen(path, "a");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(-1); }
    fprintf(f, "%lld %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %d\n", g_steps, e[0], e[1], e[2],
            e[3], e[4], ob[0], ob[1], ob[2], (int)ob[3]);
    fclose(f);
  }
}

// One step; after every nup-th step the loop's output block reads the device
// arrays (sop.cu:244-252: iup counts steps from 1 and the block runs when
// iup % nup == 0), so the mirrors are filled first.
void underdamped_iteration() {
  sop_check(sop_step(g_ctx, 1), "sop_step");
  ++g_steps;
  if (nup > 0 && g_steps % nup == 0) refresh_mirrors();
}
