// C-ABI access to the reference's own routines, for pinning the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Linked with the reference's unmodified sources
// (global.cpp, param.cpp, io.cpp, misc.cpp, random_generator.cpp, energy.cu,
// sop.cu, GPUvars.cu) by oracle/build_ref.sh, into
//   oracle/_ref/libsopref.so      sop.cu with its host list filters; the
//                                 functions below marked "host" run without a
//                                 GPU (device arrays stand on host buffers)
//   oracle/_ref/libsopref_gpu.so  sop.cu as it ships (CUDPP-based GPU list
//                                 drivers); the "device" functions need a GPU
// It drives the reference's file loader (io.cpp:112-259), FP32 host energies
// (energy.cu:194-225, 278-307, 369-442), observables (sop.cu:528-611), its
// list drivers (sop.cu:924-1262, 1351-1448, 1452-1620, 1707-1823) and its force
// kernels through force_eval (energy.cu:81-150).
#include <cstring>
#include <cstdlib>
#include "global.h"
#include "energy.h"
#include "io.h"
#include "param.h"
#include "sop.h"
#include "GPUvars.h"

extern "C" {

void ref_host_copies(int on);  // oracle/ref_link_wraps.cpp

// Resets the reference's defaults (param.cpp:8-119).
void ref_init_defaults() { alloc_arrays(); }

// Runs one `load <what> <path>;` command of the reference's input script
// (sop.cu:64-67 -> io.cpp:112).  what: bonds | angles | vdw | init.
void ref_load(const char* what, const char* path) {
  std::strcpy(cmd[1], "load");
  std::strcpy(opt[1], what);
  std::strcpy(opt[2], path);
  opt_ptr[1] = 1;
  opt_ptr[2] = 3;
  load(1);
}

void ref_sizes(int* out) {
  out[0] = nbead; out[1] = nbnd; out[2] = nang; out[3] = ncon_att; out[4] = ncon_rep;
  out[5] = nil_att; out[6] = nil_rep;
}

// Copies the loaded topology out with 0-based indices and explicit types.
void ref_topology(int* bi, int* bj, float* br0, int* ai, int* ak, int* nat_i, int* nat_j,
                  int* nat_ti, int* nat_tj, float* nat_r0, int* rep_i, int* rep_j, int* rep_ti,
                  int* rep_tj) {
  for (int b = 0; b < nbnd; ++b) {
    bi[b] = ibead_bnd[b] - 1; bj[b] = jbead_bnd[b] - 1; br0[b] = pdb_dist[b];
  }
  for (int a = 0; a < nang; ++a) { ai[a] = ibead_ang[a] - 1; ak[a] = kbead_ang[a] - 1; }
  for (int c = 0; c < ncon_att; ++c) {
    nat_i[c] = GET_IDX(idx_bead_lj_nat[c].x) - 1;
    nat_j[c] = GET_IDX(idx_bead_lj_nat[c].y) - 1;
    nat_ti[c] = GET_TYPE(idx_bead_lj_nat[c].x);
    nat_tj[c] = GET_TYPE(idx_bead_lj_nat[c].y);
    nat_r0[c] = lj_nat_pdb_dist[c];
  }
  for (int c = 0; c < ncon_rep; ++c) {
    rep_i[c] = GET_IDX(idx_bead_lj_non_nat[c].x) - 1;
    rep_j[c] = GET_IDX(idx_bead_lj_non_nat[c].y) - 1;
    rep_ti[c] = GET_TYPE(idx_bead_lj_non_nat[c].x);
    rep_tj[c] = GET_TYPE(idx_bead_lj_non_nat[c].y);
  }
}

void ref_positions(float* pos_out, float* unc_out) {
  for (int i = 0; i < nbead; ++i) {
    pos_out[3 * i] = pos[i].x; pos_out[3 * i + 1] = pos[i].y; pos_out[3 * i + 2] = pos[i].z;
    unc_out[3 * i] = unc_pos[i].x; unc_out[3 * i + 1] = unc_pos[i].y;
    unc_out[3 * i + 2] = unc_pos[i].z;
  }
}

void ref_set_state(const float* unc, const float* v) {
  for (int i = 0; i < nbead; ++i) {
    unc_pos[i].x = unc[3 * i]; unc_pos[i].y = unc[3 * i + 1]; unc_pos[i].z = unc[3 * i + 2];
    if (v) { vel[i].x = v[3 * i]; vel[i].y = v[3 * i + 1]; vel[i].z = v[3 * i + 2]; }
  }
}

// Installs explicit pair lists (0-based, all beads of type 1) as the current
// pair lists the host energy reads (energy.cu:381-438).
void ref_set_pair_lists(int natt, const int* ai, const int* aj, const float* r0, int nrep,
                        const int* ri, const int* rj) {
  for (int p = 0; p < natt; ++p) {
    idx_pair_list_att[p].x = COMBINE(1, ai[p] + 1);
    idx_pair_list_att[p].y = COMBINE(1, aj[p] + 1);
    pl_lj_nat_pdb_dist[p] = r0[p];
  }
  for (int p = 0; p < nrep; ++p) {
    idx_pair_list_rep[p].x = COMBINE(1, ri[p] + 1);
    idx_pair_list_rep[p].y = COMBINE(1, rj[p] + 1);
  }
  nil_att = natt;
  nil_rep = nrep;
}

// The reference's host energy terms: e_bnd, e_ang_ss, e_vdw_rr_att, e_vdw_rr_rep.
void ref_energies(double* out) {
  fene_energy();
  soft_sphere_angular_energy();
  vdw_energy();
  out[0] = e_bnd; out[1] = e_ang_ss; out[2] = e_vdw_rr_att; out[3] = e_vdw_rr_rep;
}

// The reference's observables for the underdamped path: Q, rgsq, kinT, contct_nat.
void ref_observables(double* out) {
  sim_type = 1;
  FLOAT3* incr = new FLOAT3[nbead];
  calculate_observables(incr);
  delete[] incr;
  out[0] = Q; out[1] = rgsq; out[2] = kinT; out[3] = contct_nat;
}

// The reference's host Gaussian deviates (random_generator.cpp:83-143) for a
// given `set run` value (param.cpp:274-279).
void ref_gasdev(int run_id, int count, double* out) {
  generator.set_seed(-100 - run_id);
  for (int k = 0; k < count; ++k) out[k] = generator.gasdev();
}

// Wrapped coordinates (the reference's pos array).
void ref_set_pos(const float* p) {
  for (int i = 0; i < nbead; ++i) {
    pos[i].x = p[3 * i]; pos[i].y = p[3 * i + 1]; pos[i].z = p[3 * i + 2];
  }
}

// The reference's output writers on the current state: trajectory frames
// (record_traj), coordinate and velocity files (save_coords, save_vels),
// io.cpp:261-381.
void ref_write_outputs(const char* traj, const char* traj_unc, const char* coord,
                       const char* unccoord, const char* vels) {
  record_traj(const_cast<char*>(traj), const_cast<char*>(traj_unc));
  save_coords(const_cast<char*>(coord), const_cast<char*>(unccoord));
  save_vels(const_cast<char*>(vels));
}

// One line of the reference's progress file for step istep (the sprintf of
// underdamped_ctrl, sop.cu:256-259) after the energies and observables
// above; rna_etot as energy_eval forms it (energy.cu:75).
void ref_update_line(double istep, char* out, int cap) {
  rna_etot = e_bnd + e_ang_ss + e_vdw_rr;
  snprintf(out, cap, "%.0lf %f %f %f %f %f %f %f %f %f %d %f", istep, T, kinT, e_bnd, e_ang_ss,
           e_vdw_rr_att, e_vdw_rr_rep, e_vdw_rr, rna_etot, Q, contct_nat, rgsq);
}

// Runs one `set <key> <value>;` command of the reference's input script
// (sop.cu:70-73 -> set_params, param.cpp:233-394).
void ref_set(const char* key, const char* value) {
  std::strcpy(cmd[1], "set");
  std::strcpy(opt[1], key);
  std::strcpy(opt[2], value);
  opt_ptr[1] = 1;
  opt_ptr[2] = 3;
  set_params(1);
}

// ---- list drivers ---------------------------------------------------------

// host: points the device arrays the host list filters stage through
// (dev_unc_pos, dev_idx_neighbor_list_*, dev_nl_lj_nat_pdb_dist) at host
// buffers sized as alloc_GPU_arrays sizes them (GPUvars.cu:105-130), and turns
// every cudaMemcpy into a host copy.  Call after the loads.
void ref_host_lists_prepare() {
  ref_host_copies(1);
  unc_pos_size = nbead * sizeof(FLOAT3);
  pos_size = unc_pos_size;
  vel_size = unc_pos_size;
  dev_unc_pos = new FLOAT3[nbead];
  dev_pos = new FLOAT3[nbead];
  dev_vel = new FLOAT3[nbead];
  dev_idx_neighbor_list_att = new ushort2[ncon_att > 0 ? ncon_att : 1];
  dev_nl_lj_nat_pdb_dist = new PDB_FLOAT[ncon_att > 0 ? ncon_att : 1];
  dev_idx_neighbor_list_rep = new ushort2[ncon_rep > 0 ? ncon_rep : 1];
  std::memcpy(dev_unc_pos, unc_pos, unc_pos_size);
}

// device: the reference's device set-up from the loaded globals, as
// underdamped_ctrl does it (sop.cu:133-140): alloc_GPU_arrays
// (GPUvars.cu:99-231), alloc_cudpp (GPUvars.cu:232-298), setup_rng
// (GPUvars.cu:430-453).
void ref_device_setup(unsigned long long seed) {
  alloc_GPU_arrays();
  alloc_cudpp();
  setup_rng(seed, 0);
}

// host or device: uploads the host coordinates and velocities to the device
// arrays (the H2D copies of alloc_GPU_arrays and load_coords).
void ref_upload_state() {
  cudaMemcpy(dev_unc_pos, unc_pos, unc_pos_size, cudaMemcpyHostToDevice);
  cudaMemcpy(dev_pos, pos, pos_size, cudaMemcpyHostToDevice);
  cudaMemcpy(dev_vel, vel, vel_size, cudaMemcpyHostToDevice);
}

// host or device: update_neighbor_list followed by update_pair_list, as the
// set-up of underdamped_ctrl calls them (sop.cu:143-147).  The neighbour list
// is copied to the host arrays before the pair-list driver reorders the device
// buffer it shares with the pair list; the pair list after it.  counts
// receives nnl_att, nnl_rep, nil_att, nil_rep.
void ref_update_lists(long long* counts) {
  update_neighbor_list();
  cudaMemcpy(idx_neighbor_list_att, dev_idx_neighbor_list_att, nnl_att * sizeof(ushort2),
             cudaMemcpyDeviceToHost);
  cudaMemcpy(nl_lj_nat_pdb_dist, dev_nl_lj_nat_pdb_dist, nnl_att * sizeof(PDB_FLOAT),
             cudaMemcpyDeviceToHost);
  cudaMemcpy(idx_neighbor_list_rep, dev_idx_neighbor_list_rep, nnl_rep * sizeof(ushort2),
             cudaMemcpyDeviceToHost);
  update_pair_list();
  cudaMemcpy(idx_pair_list_att, dev_idx_pair_list_att, nil_att * sizeof(ushort2),
             cudaMemcpyDeviceToHost);
  cudaMemcpy(pl_lj_nat_pdb_dist, dev_pl_lj_nat_pdb_dist, nil_att * sizeof(PDB_FLOAT),
             cudaMemcpyDeviceToHost);
  cudaMemcpy(idx_pair_list_rep, dev_idx_pair_list_rep, nil_rep * sizeof(ushort2),
             cudaMemcpyDeviceToHost);
  counts[0] = nnl_att; counts[1] = nnl_rep; counts[2] = nil_att; counts[3] = nil_rep;
}

// Copies one list of the last ref_update_lists as 0-based (i, j) pairs in the
// reference's order, with r0 for the attractive lists (r0 may be NULL).
// which: 0 attractive NL, 1 repulsive NL, 2 attractive PL, 3 repulsive PL.
void ref_list_copy(int which, int* i_out, int* j_out, float* r0_out) {
  const ushort2* src = which == 0 ? idx_neighbor_list_att : which == 1 ? idx_neighbor_list_rep
                     : which == 2 ? idx_pair_list_att : idx_pair_list_rep;
  const PDB_FLOAT* r0 = which == 0 ? nl_lj_nat_pdb_dist : which == 2 ? pl_lj_nat_pdb_dist : nullptr;
  const int n = which == 0 ? nnl_att : which == 1 ? nnl_rep : which == 2 ? nil_att : nil_rep;
  for (int k = 0; k < n; ++k) {
    i_out[k] = GET_IDX(src[k].x) - 1;
    j_out[k] = GET_IDX(src[k].y) - 1;
    if (r0 && r0_out) r0_out[k] = r0[k];
  }
}

// device: force_eval (energy.cu:81-150) -- clear_forces, random_force and the
// four force kernels -- on the current device pair lists at the current T;
// the device forces are copied to out (3 floats per bead).
void ref_force_eval(float* out) {
  force_eval();
  cudaMemcpy(force, dev_force, nbead * sizeof(float3), cudaMemcpyDeviceToHost);
  for (int i = 0; i < nbead; ++i) {
    out[3 * i] = force[i].x; out[3 * i + 1] = force[i].y; out[3 * i + 2] = force[i].z;
  }
}

}  // extern "C"
