/*
 * sop_gpu.h -- C ABI of libsopgpu.so, the GB300 (sm_103a) SOP engine.
 *
 * The reference (samchogroup/SOP) has no plugin API: its device side is a set
 * of free functions over process globals (energy.h:13-24, sop.h:23-60,
 * GPUvars.h:148-152).  This header is the boundary that replaces that device
 * side.  Plain pointers and sizes only; every call returns an int status
 * (SOP_OK = 0).  Host pointers are borrowed for the duration of a call.
 *
 * One context is one CUDA stream on one device.  A context holds one or more
 * independent molecules (trajectories); the reference's plain path is a
 * context with one molecule, the batched ensemble a context with many.  Calls
 * on one context are not thread-safe; separate contexts may run on separate
 * host threads.
 *
 * Indices are 0-based.  The reference stores 1-based 14-bit bead indices with
 * a 2-bit type (global.h:51-67); the engine keeps untyped indices and a
 * per-bead type array: a molecule holds up to 65,535 beads (the reference,
 * 16,383), a context any number of molecules.
 */
#ifndef SOP_GPU_H
#define SOP_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (the reference calls exit(-1) instead: energy.cu:149,165,
 * sop.cu:1002-1006, 1257-1261). */
enum {
  SOP_OK = 0,
  SOP_ERR_ARG = 1,        /* invalid argument or call order */
  SOP_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  SOP_ERR_ALLOC = 3,      /* device allocation failed */
  SOP_ERR_CAPACITY = 4,   /* a list outgrew its capacity and could not be regrown */
  SOP_ERR_MOLECULE = 5,   /* a molecule stopped: FENE bond beyond R0 or a non-finite value */
  SOP_ERR_BUDGET = 6,     /* admission refused: the HBM budget is exhausted */
  SOP_ERR_NOT_FOUND = 7   /* unknown molecule id */
};

/* Per-molecule status bits (sop_molecule_status). */
enum {
  SOP_MOL_FENE_RANGE = 1, /* |r - r0| >= R0 on some bond: log(1 - dev^2/R0^2) undefined */
  SOP_MOL_NONFINITE = 2,  /* a force or coordinate became NaN/Inf */
  SOP_MOL_DONE = 4        /* reached its step budget */
};

/*
 * Force field, integrator and list parameters (the reference's globals set by
 * alloc_arrays and set_params, param.cpp:8-119, 233-394).
 *
 * List cut-offs: a positive *_fac selects the reference's factor mode, where
 * the cut-off is fac * r0 for native pairs and fac * sigma_rep for non-native
 * pairs (sop.cu:746-749, 815-818, 861-864, 910-913: 3.2 for the neighbour
 * list, 2.5 for the pair list); *_fac <= 0 selects an absolute cut-off of
 * *_abs Angstrom.  Membership is d^2 < rcut^2, with d^2 formed in FP32 as the
 * reference's host filters do.
 *
 * Cadence: the neighbour list is rebuilt before step n when n % nnlup == 0
 * (sop.cu:200-225), the pair list when n % nplup == 0 or after a neighbour-list
 * rebuild (the reference rebuilds it every step, nplup = 1, sop.cu:227-232).
 */
typedef struct sop_params {
  double k_bnd;       /* FENE k, kcal/mol/A^2 (param.cpp:14) */
  double R0;          /* FENE R0, A (param.cpp:15) */
  double eps_ss;      /* i,i+2 soft-sphere epsilon (param.cpp:37) */
  double sigma_ss;    /* i,i+2 soft-sphere sigma, A (param.cpp:35) */
  double eps_rep;     /* non-native repulsion epsilon (energy.cu:15-19) */
  double boxl;        /* periodic box length, A (param.cpp:97) */
  double h;           /* time step, tau_L (param.cpp:104, set t_step) */
  double zeta;        /* friction, 1/tau_L (param.cpp:100) */
  double nl_att_fac, nl_att_abs, nl_rep_fac, nl_rep_abs;
  double pl_att_fac, pl_att_abs, pl_rep_fac, pl_rep_abs;
  int nnlup;          /* neighbour-list cadence, steps (param.cpp:103) */
  int nplup;          /* pair-list cadence, steps */
  int rep6;           /* 0: eps (s^12/r^12 + s^6/r^6) as energy.cu:436-437; 1: eps (s/r)^6 */
  int device;         /* CUDA device ordinal (set device, param.cpp:387-390) */
  int graph_steps;    /* steps per captured CUDA graph (0: the engine's default) */
  int lanes_per_bead; /* 0: autotuned; else 2, 4, 8 or 16 (others: SOP_ERR_ARG) */
  unsigned long long seed; /* Philox key (replaces setup_rng's seed, GPUvars.cu:417-453) */
  int integrator;     /* 0: underdamped Langevin (sop.cu:421-462); 1: overdamped,
                         x += (h / zeta) f with f = F + noise (sop.cu:487-521,
                         a5 = h / zeta, param.cpp:110); velocities stay zero */
  int step_split;     /* form of the step: 1 one kernel, 2 a force kernel and a
                         finish kernel, 3 every step between two list rebuilds
                         in one cooperative launch (a device-wide barrier
                         between steps), 4 the same in one block of 1,024
                         threads (block barriers; tried by the tuner for
                         contexts of up to 2,048 bead slots), 0 chosen by
                         timing at commit (served contexts: 2).  Every form
                         gives the same bits. */
  int step_window;    /* shared-memory window of the step, in beads: each step
                         block stages the coordinates of its beads' molecules
                         (up to this many beads) and gathers partners from
                         there.  0 chosen by timing at commit, < 0 none, at
                         most 12288.  Served contexts use none.  Every window
                         gives the same bits. */
  int step_buckets;   /* per-size-bucket tiles of a batched context: molecules
                         of < 200, 200-599 and >= 600 beads each get the lanes
                         per bead and the form the tuner chose for their
                         bucket, in per-molecule tiles of one launch.  0: used
                         when the tuner times it faster than the best
                         whole-context step, 1: always (lanes and form must
                         be left to the tuner), < 0: never.  Same bits. */
  int nl_rows;        /* initial length of the neighbour-list rows, entries
                         (rounded up to a multiple of 32); 0: sized for the
                         densest synthetic globules (1.3 x 6e-3 beads / A^3
                         within the largest cut-off, at most the largest
                         molecule).  A row that outgrows it regrows the rows,
                         at commit, at an upload or mid-run. */
} sop_params;

/* Fills *p with the reference's defaults and the factor-mode list cut-offs. */
void sop_params_default(sop_params* p);

/*
 * One molecule: what the reference's bonds/angles/vdw/init files hold
 * (io.cpp:112-259).  Non-native pairs are implicit: every pair with
 * |i - j| > 2 that is not a native contact (the content of the reference's
 * idx_bead_lj_non_nat, io.cpp:216-225).
 */
typedef struct sop_molecule {
  int nbead;
  int nbnd;  const int* bond_i; const int* bond_j; const float* bond_r0;
  int nang;  const int* ang_i;  const int* ang_k;          /* soft sphere on (i, k) */
  int nnat;  const int* nat_i;  const int* nat_j; const float* nat_r0;
  const float* nat_eps;        /* epsilon of the native force; NULL: 1.0 */
  const float* nat_eps_energy; /* epsilon of the native energy; NULL: nat_eps */
  const int* types;            /* per bead 1 or 2 (sigma_rep table); NULL: all 1 */
  const float* unc_pos;        /* 3*nbead unwrapped coordinates (required) */
  const float* pos;            /* 3*nbead wrapped coordinates; NULL: unc_pos */
  const float* vel;            /* 3*nbead; NULL: zero (sop.cu:117-128) */
  double T;                    /* kBT, kcal/mol (param.cpp:92, set temp) */
  unsigned int traj;           /* Philox stream id of this trajectory */
  long long nsteps;            /* step budget; < 0: unlimited */
} sop_molecule;

/* Context lifetime: replaces alloc_GPU_arrays / alloc_cudpp / setup_rng
 * (GPUvars.cu:99-293, 417-453). */
int sop_ctx_create(const sop_params* p, void** ctx);
int sop_ctx_destroy(void* ctx);

/* Stages a molecule; *mol_id receives its id.  Device state is created by
 * sop_commit. */
int sop_add_molecule(void* ctx, const sop_molecule* m, int* mol_id);

/*
 * Uploads every staged molecule, builds the neighbour and pair lists from the
 * initial coordinates and evaluates the initial forces: the set-up half of
 * underdamped_ctrl (sop.cu:133-186: alloc_GPU_arrays, setup_rng,
 * update_neighbor_list, update_pair_list, force_eval).
 */
int sop_commit(void* ctx);

/* Single-molecule convenience: sop_add_molecule + sop_commit. */
int sop_upload_topology(void* ctx, const sop_molecule* m);

/* Replaces coordinates and velocities of molecule `mol` (load_coords /
 * load_vels H2D, io.cpp:361-363, 407) and re-evaluates its forces. */
int sop_upload_state(void* ctx, int mol, const float* pos, const float* unc_pos,
                     const float* vel);

/*
 * Advances every active molecule nsteps Langevin steps: the loop body of
 * underdamped_ctrl (sop.cu:197-243) -- list rebuilds on their cadence,
 * underdamped_iteration_kernel, force_eval, update_velocities_kernel
 * (sop.cu:421-484) -- run as fused kernels in captured CUDA graphs.
 */
int sop_step(void* ctx, long long nsteps);

/*
 * sop_step without the final wait: queues nsteps steps on the context's
 * stream and returns.  A neighbour-list overflow during the queued work
 * freezes every molecule at the start of the block that overflowed;
 * sop_sync regrows the lists and re-runs the frozen steps.  Together they
 * are sop_step; apart they let a caller overlap host work or time the device
 * work alone.  The reference's loop always waits (cudaThreadSynchronize,
 * energy.cu:148).
 */
int sop_step_async(void* ctx, long long nsteps);
int sop_sync(void* ctx);

/*
 * Queues one stage of the step loop at block offset koff, for timing and
 * profiling: 0 the fused force + Langevin step kernel, 1 the pair-list
 * rebuild, 2 the neighbour-list rebuild, 3 the end-of-block step advance
 * (count = koff).  Stages launched out of the loop's order leave the
 * trajectory undefined; the loop itself is sop_step.
 */
int sop_launch_stage(void* ctx, int stage, int koff);

/* Rebuilds the neighbour lists now (update_neighbor_list, sop.cu:928-1262);
 * returns the attractive / repulsive totals over all molecules (pairs, each
 * counted once) when the pointers are non-NULL. */
int sop_update_neighbor_list(void* ctx, long long* nnl_att, long long* nnl_rep);

/* Rebuilds the pair lists from the neighbour lists (update_pair_list,
 * sop.cu:1456-1706). */
int sop_update_pair_list(void* ctx, long long* nil_att, long long* nil_rep);

/* Re-evaluates forces at the current coordinates, noise included
 * (force_eval + random_force, energy.cu:81-167). */
int sop_force_eval(void* ctx);

/*
 * Noise injection: with normals != NULL the next force evaluation uses
 * force += sqrt(2 T zeta / h) * normals[3*i + c] for every bead i of every
 * molecule (beads numbered across molecules in id order) instead of the
 * Philox stream; NULL returns to Philox.  Replaces random_force's
 * generator (energy.cu:154-188) for single-step parity checks.
 */
int sop_set_noise(void* ctx, const float* normals);

/* Copies molecule `mol`'s current state to host arrays of 3*nbead floats;
 * NULL pointers are skipped (the D2H reads of sop.cu:252-263). */
int sop_download(void* ctx, int mol, float* pos, float* unc_pos, float* vel, float* force);

/*
 * Copies molecule `mol`'s lists as (i, j) pairs with i < j, 0-based.
 * which: 0 attractive neighbour list, 1 repulsive neighbour list,
 *        2 attractive pair list,      3 repulsive pair list.
 * cap is the capacity of i_out / j_out (and r0_out for the attractive lists,
 * NULL allowed); *count receives the list size even when it exceeds cap.
 */
int sop_download_list(void* ctx, int mol, int which, long long cap, int* i_out, int* j_out,
                      float* r0_out, long long* count);

/* Current list sizes over all molecules, each pair counted once:
 * out[0..3] = attractive NL, repulsive NL, attractive PL, repulsive PL
 * (the reference's nnl_att, nnl_rep, nil_att, nil_rep globals). */
int sop_list_sizes(void* ctx, long long* out);

/* Current unwrapped coordinates of every molecule, molecules in id order,
 * 3 floats per bead, into one host array (one device-to-host copy). */
int sop_download_all(void* ctx, float* unc_pos);

/*
 * sop_download_all without the waits: queues a gather of the coordinates
 * the queued work will have reached, and their copy into unc_pos on a copy
 * stream of the context, so that the copy overlaps the steps queued after
 * it.  Returns at once (when unc_pos is page-locked host memory) with a
 * ticket.  sop_download_wait(ticket) waits for that copy; it returns
 * SOP_ERR_CAPACITY when the neighbour lists had overflowed before the
 * gather (the coordinates are then those of the frozen molecules: sop_sync
 * re-runs the frozen steps, and a new download gives the right ones).
 * unc_pos must stay valid until the wait.  Two downloads may be in flight;
 * a third waits on the device for the first one's copy.  The reference
 * reads back with blocking copies (sop.cu:252-263).
 */
int sop_download_all_async(void* ctx, float* unc_pos, long long* ticket);
int sop_download_wait(void* ctx, long long ticket);

/*
 * Energy terms of molecule `mol` on its current pair lists (energy_eval and
 * the host energies of energy.cu:69-78, 194-225, 278-307, 369-442), per-term
 * FP32 evaluation with an FP64 final sum.  terms: e_bnd, e_ang_ss,
 * e_vdw_rr_att, e_vdw_rr_rep, rna_etot.
 */
int sop_energy(void* ctx, int mol, double* terms);

/* Observables of calculate_observables (sop.cu:528-611): Q, rgsq, kinT,
 * contct_nat, with FP64 reductions. */
int sop_observables(void* ctx, int mol, double* out);

/* Molecule status bits (SOP_MOL_*) and its completed step count. */
int sop_molecule_status(void* ctx, int mol, int* status, long long* step);

/* Total device bytes held by the context, and the bytes charged to `mol`. */
int sop_memory(void* ctx, int mol, long long* ctx_bytes, long long* mol_bytes);

/* Lanes per bead the step kernel uses (chosen at sop_commit by timing 2, 4, 8
 * and 16 unless sop_params.lanes_per_bead fixed it) and the measured kernel
 * times in ms for those four candidates (0 when not tuned).  Forces are
 * bit-identical for every choice. */
int sop_tuning(void* ctx, int* lanes, float* ms);
/* The step's shape in use: lanes per bead, and its form (1 one kernel, 2 a
 * force kernel and a finish kernel, 3 persistent: the steps between two list
 * rebuilds in one cooperative launch, 4 the same in one block). */
int sop_step_form(void* ctx, int* lanes, int* form);

/* The per-size-bucket tiling of the step (sop_params.step_buckets): *tiled
 * receives 1 when the tiled step is in use; per bucket (< 200, 200-599,
 * >= 600 beads) the lanes per bead and form chosen and the beads it holds
 * (arrays of 3, NULL skips); ms[0], ms[1]: the tuned times of the tiled step
 * and of the best whole-context step (0 when not tuned). */
int sop_step_buckets(void* ctx, int* tiled, int* lanes, int* forms, long long* beads, float* ms);

/* The step's shared-memory window in beads (0: partners gathered from global
 * memory). */
int sop_step_window(void* ctx, int* wcap);

/*
 * Health check of the persistent step form's device-wide barrier (no
 * counterpart in the reference).  Runs three barriers over the persistent
 * form's grid, with `missing` arrivals that never come (0: the barriers must
 * complete), each wait limited to timeout_s seconds (at most 10).
 * *timed_out receives 1 when a wait ran out: the kernel then returns instead
 * of spinning, the context stays usable and the flag is cleared.  A timed-out
 * wait inside a step makes sop_step / sop_sync fail with SOP_ERR_CUDA.
 */
int sop_check_step_barrier(void* ctx, int missing, double timeout_s, int* timed_out);

/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work around the engine. */
int sop_stream(void* ctx, void** stream);

/*
 * Serving (continuous batching).  No counterpart in the reference, which
 * runs one molecule per process (sop.cu:13-55).  A served context holds
 * device pools sized by an HBM budget (coordinates, velocities, topology,
 * neighbour and pair lists, Philox counters are implicit) and runs jobs --
 * molecules with step budgets -- that are submitted while others run.  Each
 * sop_serve_advance round: wait for the previous round, retire finished or
 * failed jobs (results copied to the host, slots freed), admit queued jobs in
 * arrival order while their beads, topology and list rows fit the pools, then
 * queue nnlup more steps of every active job.  An admitted job starts at the
 * round's neighbour-list rebuild, so its own step count keeps the reference's
 * cadence, and its trajectory is bit-identical to the same job run alone.
 */
int sop_serve_create(const sop_params* p, long long budget_bytes, long long max_job_beads,
                     void** ctx);   /* max_job_beads <= 65,535 */
/* Queues a job (m->nsteps must be >= 0); *job receives its id. */
int sop_serve_submit(void* ctx, const sop_molecule* m, int* job);
/* Runs `rounds` rounds; returns when their work is queued on the device. */
int sop_serve_advance(void* ctx, int rounds);
/* Ids of jobs finished since the previous call (up to cap); *count receives
 * how many were written. */
int sop_serve_finished(void* ctx, int cap, int* jobs, int* count);
/* Results of a finished job: coordinates and velocities (3*nbead floats, NULL
 * skips), energy terms as sop_energy (5 doubles), SOP_MOL_* status, steps
 * completed and the seconds from submission to retirement. */
int sop_serve_result(void* ctx, int job, float* unc_pos, float* vel, double* energy,
                     int* status, long long* steps, double* latency_s);
/* out[0..7]: queued, active, finished jobs; active beads; bead capacity;
 * device bytes held; budget; the context's step clock. */
int sop_serve_stats(void* ctx, long long* out);

/*
 * Exact checkpoints.  The reference saves coordinates and velocities
 * (save_coords / save_vels, io.cpp:261-381, called from sop.cu:268-272) and
 * restarts from them; its GPU random state is not saved.  A checkpoint here
 * holds everything the following steps read: the step counter and status,
 * the coordinates of the last completed step and the look-ahead of the next,
 * velocities, increments and forces, and the molecule's neighbour- and
 * pair-list rows.  Restored into a context with the same parameters and the
 * same molecule (topology, T, trajectory id, seed), the continuation is
 * bit-identical to the run it came from.
 *
 * sop_checkpoint: buf = NULL returns the size in *size; otherwise cap bytes
 * at buf receive the checkpoint.  Plain and batched contexts.
 * sop_restore: writes a checkpoint into molecule `mol` of a committed
 * context.  The context has one step clock: the first restore into a
 * context that has not stepped sets it to the checkpoint's step, later
 * restores must carry that same step.
 */
int sop_checkpoint(void* ctx, int mol, void* buf, long long cap, long long* size);
int sop_restore(void* ctx, int mol, const void* buf, long long size);
/* Served contexts: the checkpoint of a running job (taken between rounds,
 * when its step is a multiple of nnlup), and a job that continues from one
 * (queued like sop_serve_submit; m describes the same molecule, m->nsteps is
 * the job's total step budget). */
int sop_serve_checkpoint(void* ctx, int job, void* buf, long long cap, long long* size);
int sop_serve_resume(void* ctx, const sop_molecule* m, const void* buf, long long size, int* job);

/*
 * Energy without allocation.  No counterpart in the reference: an extension
 * for callers that may not allocate device memory -- a host application whose
 * own memory manager owns every device byte, a loop that must not stall on the
 * implicit synchronisation cudaMalloc / cudaFree can bring, or an embedding
 * whose framework forbids allocations outside its pool.  The caller owns every
 * buffer below (device memory) and the output; the call only launches kernels
 * on `stream` (a cudaStream_t, NULL for the default stream) and returns
 * without waiting.
 *
 * Layout: flat arrays of 0-based bead indices, one entry per term -- bonds
 * (bond_i, bond_j) with their native lengths, i,i+2 angle pairs (ang_i,
 * ang_k), native pairs (att_i, att_j) with r0 and the epsilon of the native
 * ENERGY (att_eps; NULL: 1.0 for every pair), non-native pairs (rep_i,
 * rep_j) -- and a separate per-bead type array (1 or 2, selecting sigma_rep;
 * NULL: all 1).  Every index must lie in [0, nbead) and every type be 1 or 2:
 * an entry that breaks this is not evaluated and turns its term and rna_etot
 * into NaN.  terms receives 5 doubles as sop_energy: e_bnd, e_ang_ss,
 * e_vdw_rr_att, e_vdw_rr_rep, rna_etot.
 *
 * Limit: at most SOP_ENERGY_NOALLOC_MAX_ITEMS list entries in total (bonds +
 * angles + native + non-native pairs); larger inputs fail with
 * SOP_ERR_CAPACITY before any launch.  The per-block partial sums live in one
 * fixed 128 KiB device array that every GPU loading the library holds until
 * the process exits.  Every call looks up that array's device address
 * (cudaGetSymbolAddress) in the caller's current device and context; the first
 * call in a context also loads the library's device code there, so make it
 * before any stream capture.  Every call shares the array and overwrites the
 * part it uses, so calls that overlap on the GPU (different streams, or
 * different host threads on one device) race; serialise them.
 */
#define SOP_ENERGY_NOALLOC_MAX_ITEMS 4194304LL
typedef struct sop_energy_lists {
  int nbead;  const float* unc_pos;                 /* 3*nbead floats */
  const int* types;                                 /* nbead, 1 or 2; NULL: all 1 */
  int nbnd;   const int* bond_i; const int* bond_j; const float* bond_r0;
  int nang;   const int* ang_i;  const int* ang_k;
  int natt;   const int* att_i;  const int* att_j;  const float* att_r0; const float* att_eps;
  long long nrep; const int* rep_i; const int* rep_j;
} sop_energy_lists;
int sop_energy_noalloc(const sop_params* p, const sop_energy_lists* l, double* terms, void* stream);
/* Message of the calling thread's last sop_energy_noalloc failure. */
const char* sop_energy_noalloc_error(void);

/* Last error message of the context (or of the library when ctx is NULL). */
const char* sop_last_error(void* ctx);

#ifdef __cplusplus
}
#endif
#endif /* SOP_GPU_H */
