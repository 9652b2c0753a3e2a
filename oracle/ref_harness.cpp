// C-ABI access to the reference's own host routines, for pinning the oracle.
//
// TEST INFRASTRUCTURE ONLY.  Linked with the reference's unmodified sources
// (global.cpp, param.cpp, io.cpp, misc.cpp, random_generator.cpp, energy.cu,
// sop.cu, GPUvars.cu) into oracle/_ref/libsopref.so by oracle/build_ref.sh.
// Nothing here touches a GPU: it drives the reference's file loader
// (io.cpp:112-259), FP32 host energies (energy.cu:194-225, 278-307, 369-442)
// and observables (sop.cu:528-611) on host arrays.
#include <cstring>
#include "global.h"
#include "energy.h"
#include "io.h"
#include "param.h"
#include "sop.h"

extern "C" {

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

}  // extern "C"
