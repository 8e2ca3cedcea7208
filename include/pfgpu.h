/*
 * pfgpu.h - C ABI of the GB300 (sm_103a) phase-field step library libpfgpu.so
 *
 * Drop-in replacement for the time step of the reference program var_diff.x
 * (smjim/phase-field-microstructure-evolution):
 *   - the loop body src/var_diff.f90:474-1118 (14 timed phases + statistics),
 *   - the FFT wrappers src/f_trans.f90:1-15 and src/inv_trans.f90:1-13,
 *   - the wavenumber tables src/k_space.f90:4-67.
 * The reference calls these as implicit-interface Fortran externals with
 * everything passed by reference (src/var_diff.f90:565,635,869-870,944,964,
 * 994,1003-1008,1045 and :466); this header offers
 *   (1) a step-level API (pf_create / pf_set_fields / pf_step / pf_get_fields /
 *       pf_destroy) that replaces the whole loop body on one GPU, and
 *   (2) compatibility shims with the exact Fortran signatures of f_trans,
 *       inv_trans and k_space for a single-rank (ist = 1, ien = N) layout.
 * Plain pointers and sizes only; every call returns 0 on success and a
 * negative PF_E* code on failure, with a message from pf_last_error().
 * Host arrays belong to the caller; device buffers belong to the run.
 */
#ifndef PFGPU_H
#define PFGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PFGPU_ABI_VERSION 1

/* status codes */
#define PF_OK 0
#define PF_EINVAL (-1)     /* bad argument / unsupported size */
#define PF_ECUDA (-2)      /* CUDA runtime error (message has details) */
#define PF_ENOMEM (-3)     /* device allocation failed */
#define PF_ENONFINITE (-4) /* a step produced NaN/Inf (fields left as computed) */
#define PF_EIO (-5)        /* file I/O error */
#define PF_EBUSY (-6)      /* a wait ran out of time (the work goes on) */

/* mobility forms of the concentration equation */
#define PF_MOB_REFERENCE 0 /* mob = D_L + 2(1 - sum phi_i^2) D_gb  (src/var_diff.f90:893-898) */
#define PF_MOB_C1MC 1      /* mob = D_L (1 + c (1 - c)) */

/* arithmetic of the step */
#define PF_FP32_FUSED 32 /* fused sm_103a kernels, FP32 fields and FFTs */
#define PF_FP64_PLAIN 64 /* plain FP64 path: cuFFT + one kernel per reference phase */

/* Coefficients of one run; names and meaning follow input.txt
 * (src/var_diff.f90:104-121). dx, dy, dz are not used by the reference step. */
typedef struct pf_config {
  int nx, ny, nz;        /* Nx, Ny, Nz */
  int var;               /* number of order parameters (last one = precipitate) */
  double t_step;         /* dt */
  double grad_coeff_phi; /* kappa_phi */
  double grad_coeff_c;   /* kappa_c */
  double D_S;            /* read but unused by the reference step */
  double D_L;            /* bulk mobility, also D_mean (src/var_diff.f90:916) */
  double D_gb;           /* grain-boundary mobility */
  double mob_phi;        /* Allen-Cahn mobility L */
  double sigma_1, sigma_2;
  double am, ap, con_0_mat, con_0_ppt;
  int mobility;          /* PF_MOB_* */
  int precision;         /* PF_FP32_FUSED or PF_FP64_PLAIN */
  int device;            /* CUDA device ordinal */
  int reserved[5];
} pf_config;

/* Diagnostics of one step.  f_int, f_eta, f_ch and the statistics c_min,
 * c_max, phi_min (min over cells of sum_i phi_i^2) and phi_P_max describe the
 * fields at the START of the step: exactly the values that var_diff.f90
 * writes to summary.dat for that step (:1058-1074, statistics lagged by one
 * step, :1076-1118).  mass = sum_cells c at the start of the step. */
typedef struct pf_diag {
  int step; /* 1-based step number since pf_create / the last pf_set_fields */
  int nonfinite;
  double f_int, f_eta, f_ch, e_tot;
  double c_max, c_min, phi_min, phi_P_max;
  double mass;
} pf_diag;

typedef struct pf_run pf_run;

/* ---- step-level API (replaces src/var_diff.f90:474-1118) ---------------- */

/* Create a run on cfg->device: validates the sizes, allocates the resident
 * state and builds the FP64 wavenumber/twiddle tables.  Supported grids on
 * the fused FP32 path: Nx, Ny, Nz in {16, 32, 64, 80, 96, 102, 128, 160,
 * 200, 256} (the reference's weak-scaling grids included; every
 * (Ny, Nz) pair with Ny == Nz plus the non-cubic pairs listed by
 * pf_supported_shape), 1 <= var <= 255 as long as var+1 field rows of the x
 * pass fit in shared memory (var <= 129 at Nx = 96, 97 at 128, 195 at 256).
 * The FP64 path takes any even Nx. */
int pf_create(const pf_config* cfg, pf_run** out);

/* 1 if (nx, ny, nz, var) can run on the given precision path, else 0. */
int pf_supported_shape(int nx, int ny, int nz, int var, int precision);

/* Upload fields from host arrays in Fortran order: phi(var, x, y, z) with var
 * fastest (src/var_diff.f90:154) and con(x, y, z) (:143), REAL*8. Resets the
 * step counter. */
int pf_set_fields(pf_run* run, const double* phi_aos, const double* con);

/* Advance nsteps steps.  diag (may be NULL) receives nsteps records. Returns
 * PF_ENONFINITE if any step produced a non-finite value. */
int pf_step(pf_run* run, int nsteps, pf_diag* diag);

/* Download fields into host arrays in the pf_set_fields layout. */
int pf_get_fields(pf_run* run, double* phi_aos, double* con);

/* Release device memory and the run. */
int pf_destroy(pf_run* run);

/* Last error message of the calling thread ("" if none). */
const char* pf_last_error(void);

/* ---- batched API: many same-shape runs advanced by one set of launches --- */
typedef struct pf_batch pf_batch;
int pf_batch_create(const pf_config* cfgs, int nruns, pf_batch** out);
int pf_batch_set_fields(pf_batch* b, int run, const double* phi_aos, const double* con);
/* diag (may be NULL) receives nruns * nsteps records, run-major. */
int pf_batch_step(pf_batch* b, int nsteps, pf_diag* diag);
int pf_batch_get_fields(pf_batch* b, int run, double* phi_aos, double* con);
int pf_batch_destroy(pf_batch* b);

/* ---- a run's error against the FP64 GPU path -------------------------------
 * The same start stepped nsteps times on the fused FP32 path and on the plain
 * FP64 path (cuFFT + one kernel per phase of src/var_diff.f90:556-1050, held
 * to the FP64 CPU restatement at 1e-10 by the tests); the fields are compared
 * on the device: max-abs and L2 difference relative to the FP64 fields'
 * max-abs and L2 norm, for all order parameters together and for c.  Holds
 * both runs' memory while it works. */
typedef struct pf_error_report {
  int steps, pad;
  double phi_max_abs_rel, phi_l2_rel, c_max_abs_rel, c_l2_rel;
} pf_error_report;
int pf_check_fp64(const pf_config* cfg, const double* phi_aos, const double* con, int nsteps, pf_error_report* out);

/* ---- serving: continuous batching of independent runs on one GPU --------
 * The reference runs a parameter study as one SLURM job per run
 * (tests/run_phase_sim.py:130-172); a pf_server takes the runs as requests in
 * one process.  A worker thread admits queued requests as the resident runs
 * leave room in the device-memory budget and in max_active; waiting requests
 * of the same grid, var and mobility class are admitted together as one
 * batch and every batch steps on its own stream.  Batches that fill the GPU by
 * themselves (runs x cells x (var+1) >= 2^24) take turns, oldest admitted
 * first; smaller batches run beside them on high-priority streams.  A run
 * leaves as soon as its own step count is reached.  Results do not depend on what else is running (per-run
 * reductions, no shared state).  Fused FP32 path only. */
typedef struct pf_server pf_server;
typedef struct pf_server_config {
  int device;
  int max_active;          /* runs resident at once (0: 64) */
  double hbm_budget_bytes; /* device memory the server's runs may hold (0: 80 % of free memory at create) */
  int chunk_steps;         /* steps a batch is given at a time (0: 128; larger values are cut to 512,
                              so that the records of the two chunks kept in flight fit the per-run
                              ring of 1024 records) */
  int reserved[5];
} pf_server_config;
typedef struct pf_request_times {
  double queued_s; /* submit -> admitted */
  double run_s;    /* admitted -> finished */
  double total_s;  /* submit -> finished */
} pf_request_times;
#define PF_REQ_QUEUED 0
#define PF_REQ_RUNNING 1
#define PF_REQ_DONE 2
#define PF_REQ_FAILED 3
int pf_server_create(const pf_server_config* cfg, pf_server** out);
/* Queue a run of nsteps steps from the given fields (copied; layout of
 * pf_set_fields).  *id identifies the request. */
int pf_server_submit(pf_server* s, const pf_config* cfg, const double* phi_aos, const double* con, int nsteps,
                     long long* id);
/* State of a request (PF_REQ_*). */
int pf_server_poll(pf_server* s, long long id, int* state);
/* Wait for a request (timeout_s < 0: no limit; PF_EBUSY when it runs out),
 * then copy its final fields (may be NULL), the record of its last step and
 * its times, and forget it.  A failed request returns its error code. */
int pf_server_wait(pf_server* s, long long id, double timeout_s, double* phi_aos, double* con, pf_diag* last,
                   pf_request_times* times);
/* Finish the work in flight, fail what is still queued, release everything. */
int pf_server_destroy(pf_server* s);
/* Message of the last failed pf_server_* call of the calling thread. */
const char* pf_server_last_error(void);

/* ---- independent runs over the node's GPUs (no collective) ----------------
 * The reference fans a study out as one SLURM job per run
 * (tests/scaling_tests.py:88-124, tests/run_phase_sim.py:130-172).  Here runs
 * never exchange data, so the GPUs of a node share the work only through
 * placement: one pf_server per device, each request sent to the device with
 * the least outstanding work (cell-steps x P of its unfinished requests). */
/* Visible CUDA devices (0 without a GPU). */
int pf_device_count(void);
/* Work of a run: nx ny nz var nsteps (cell-steps x P). */
double pf_run_work(const pf_config* cfg, int nsteps);
/* Online placement: index of the smallest outstanding[d] (ties: lowest d). */
int pf_pick_device(const double* outstanding, int ndev);
/* Offline placement of nunits work units (LPT): largest unit first onto the
 * device with the least work so far.  device_of_unit[u] in [0, ndev); load
 * (may be NULL) receives the work per device. */
int pf_place_units(const double* work, int nunits, int ndev, int* device_of_unit, double* load);
typedef struct pf_pool pf_pool;
typedef struct pf_pool_config {
  int ndevices;            /* devices to use (0: every visible device) */
  const int* devices;      /* their ordinals (NULL: 0 .. ndevices-1) */
  pf_server_config server; /* settings of every device's server (its device field is ignored) */
} pf_pool_config;
int pf_pool_create(const pf_pool_config* cfg, pf_pool** out);
int pf_pool_devices(pf_pool* p);
/* As pf_server_submit; *device (may be NULL) receives the chosen ordinal. */
int pf_pool_submit(pf_pool* p, const pf_config* cfg, const double* phi_aos, const double* con, int nsteps,
                   long long* id, int* device);
/* As pf_server_wait. */
int pf_pool_wait(pf_pool* p, long long id, double timeout_s, double* phi_aos, double* con, pf_diag* last,
                 pf_request_times* times);
int pf_pool_destroy(pf_pool* p);
const char* pf_pool_last_error(void);

/* ---- Fortran compatibility shims (single rank, FP64, whole grid) ---------
 * Same argument lists as the reference subroutines, all by reference, with
 * gfortran/ifort-on-Linux name mangling.  ist = (1,1,1), ien = (Nx,Ny,Nz);
 * the complex array uses P3DFFT's transposed (STRIDE1) order with
 * fst = (1,1,1), fen = (Nz, Ny, Nx/2+1): dimension 1 = z, 2 = y, 3 = kx.
 * They run on the FP64 GPU path (device 0 unless pf_shim_device is called).
 */
/* f_trans.f90:1   subroutine f_trans(in, out, Nx, Ny, Nz, ist, ien, fst, fen) */
void f_trans_(const double* in, double* out_cplx, const int* Nx, const int* Ny, const int* Nz,
              const int* ist, const int* ien, const int* fst, const int* fen);
/* inv_trans.f90:1 subroutine inv_trans(in, out, ist, ien, fst, fen) */
void inv_trans_(const double* in_cplx, double* out, const int* ist, const int* ien, const int* fst,
                const int* fen);
/* k_space.f90:4   subroutine k_space(Nx, Ny, Nz, fst, fen, kf, kf_sq, kf_4) */
void k_space_(const int* Nx, const int* Ny, const int* Nz, const int* fst, const int* fen, double* kf,
              double* kf_sq, double* kf_4);
/* select the device used by the shims; returns PF_OK or an error code */
int pf_shim_device(int device);

/* ---- host-side helpers of the drop-in driver (no GPU needed) ------------- */

/* The reference's RNG ran_2 (src/ran_2.f90:1-40) with its saved state kept in
 * *state (an opaque 40-int buffer zeroed by pf_ran2_init). */
typedef struct pf_ran2_state {
  int idum2, iy, iv[32];
  int initialised;
  int pad[5];
} pf_ran2_state;
void pf_ran2_init(pf_ran2_state* st);
double pf_ran2(pf_ran2_state* st, int* idum);

/* ---- diagnostics without allocation ---------------------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory (their memory belongs to another runtime's pool, they run under a
 * fixed memory cap, or they may not call cudaMalloc where they are): the
 * f_eta, f_ch, mass, c_min, c_max, phi_min and phi_P_max of the pf_step record
 * (src/var_diff.f90:685-759, :1076-1102), computed from fields the caller
 * already holds on the current device, with no allocation.
 *   fields: float [var+1][nz][ny][nx] device memory, phi_1..phi_var then c;
 *   out:    host record; f_int and e_tot are NaN (they need the transforms);
 *           nonfinite counts the cells holding a NaN or Inf value;
 *   stream: cudaStream_t or NULL; the call waits for its own work, so it is
 *           rejected (PF_EINVAL) on a stream that is being captured.
 * Scratch is a fixed 512 KiB __device__ array present on every GPU that loads
 * the library until the process exits; grids above PF_NOALLOC_MAX_CELLS are
 * rejected with PF_EINVAL.  Every call looks the array up in the current
 * context.  All calls share the scratch, so calls that overlap on the GPU
 * race. */
#define PF_NOALLOC_MAX_CELLS (256 * 256 * 256)
int pf_diag_fields_noalloc(const pf_config* cfg, const float* fields, pf_diag* out, void* stream);

/* ---- input.txt, restart files and the reference's starts (host only) -----
 * The values of src/var_diff.f90:104-121, read with Fortran list-directed
 * rules: one READ per record, blanks or commas between values, r*c repeats,
 * quoted strings, '/' ends a record early (the items after it keep their
 * previous value: set_mask bit b says which group was read), a record may
 * continue on following lines.  Lines after `start` may hold key=value pairs
 * that the reference ignores: seed, n_grains, amp_phi, amp_c, c0 (for the
 * 'noise' and 'voronoi' starts), mobility (reference|c1mc), precision (32|64),
 * microstructure (the 'polycryst' file; the reference opens a fixed path),
 * check_fp64 (steps of the start compared with the FP64 GPU path). */
typedef struct pf_input {
  int nrun, ppt_int;                       /* bits 0, 1 */
  int ppt_rad[3], N_step, ifreq;           /* bits 2, 3, 4 */
  int i_ppt, j_ppt, k_ppt, iseed;          /* bits 5, 6 */
  int grn_rad, num_ppt;                    /* bits 7, 8 */
  double c_mat, c_ppt;                     /* bits 9, 10 */
  int Nx, Ny, Nz, var;                     /* bits 11, 12 */
  double dx, dy, dz, t_step;               /* bits 13, 14 */
  double grad_coeff_phi, grad_coeff_c, D_S, D_L, D_gb, mob_phi; /* bits 15-20 */
  double sigma_1, sigma_2;                 /* bit 21 */
  double am, ap, con_0_mat, con_0_ppt;     /* bits 22, 23 */
  double gb_force;                         /* bit 24 */
  int ndim, dims[2];                       /* bits 25, 26 */
  char start[16];                          /* bit 27 (character*10 in the reference) */
  unsigned long long set_mask;
  /* key=value extensions */
  int seed, n_grains, mobility, precision; /* precision 0: fused FP32 where supported */
  double amp_phi, amp_c, c0;
  char microstructure[256];
  int check_fp64; /* > 0: report the run's error against the FP64 GPU path after this many steps */
} pf_input;

/* Message of the last failed pf_read_input / pf_*data_save / pf_ic_* call. */
const char* pf_io_last_error(void);
/* Read input.txt (src/var_diff.f90:104-121); nprocs fills dims when ndim = 1. */
int pf_read_input(const char* path, int nprocs, pf_input* in);
/* pf_config of the step from an input record (device 0). */
void pf_input_to_config(const pf_input* in, pf_config* cfg);

/* data_save.NNNN / data_rerun.NNNN (src/var_diff.f90:1134-1140, :453-458):
 * Fortran unformatted sequential, two records "ist, ien" (6 INTEGER*4) and
 * "phi, con" (REAL*8, phi(var,x,y,z) then con(x,y,z)), gfortran record
 * markers (4-byte lengths; sub-records above 2^31-9 bytes), one rank. */
int pf_write_data_save(const char* path, const pf_config* cfg, const double* phi_aos, const double* con);
int pf_read_data_save(const char* path, const pf_config* cfg, double* phi_aos, double* con);

/* The reference's starts, one rank, phi(var,x,y,z) / con(x,y,z) REAL*8.
 * 'circle' (src/var_diff.f90:373-449) draws from ran_2 with *idum and *st and
 * leaves both advanced, as the later precipitate insertion continues them. */
int pf_ic_circle(const pf_config* cfg, int grn_rad, const int* ppt_rad, int num_ppt, int* idum, double c_mat,
                 double con_0_ppt, pf_ran2_state* st, double* phi_aos, double* con);
/* 'plane' (src/var_diff.f90:252-371) */
int pf_ic_plane(const pf_config* cfg, const int* ppt_rad, int i_ppt, int j_ppt, int k_ppt, double c_mat,
                double* phi_aos, double* con);
/* 'polycryst' (src/var_diff.f90:232-250): Nx*Ny*Nz text lines "i j k ivar" */
int pf_ic_polycryst(const pf_config* cfg, const char* path, double c_mat, double* phi_aos, double* con);
/* Precipitates inserted at step ppt_int (src/var_diff.f90:479-554). */
int pf_insert_precipitates(const pf_config* cfg, const int* ppt_rad, int num_ppt, int* idum, pf_ran2_state* st,
                           double* phi_aos);
/* Fortran Ew.d edit of x into out (w+1 bytes), e.g. the e15.7 of summary.dat. */
void pf_format_e(double x, int w, int d, char* out);
/* One summary.dat record, format (i6, 8e15.7) (src/var_diff.f90:1070-1071,
 * :1161): step, f_int, f_ch, f_eta, e_tot, c_max, c_min, phi_min, phi_P_max.
 * out holds at least 128 bytes; no newline. */
void pf_format_summary(int step, const pf_diag* d, char* out);
/* gfortran list-directed output of one INTEGER*4 (width 12) or REAL*8
 * (width 25, 17 significant digits), as in time_step.dat and
 * gamma_matrix.dat; out holds at least 32 bytes. */
void pf_format_list_int(int v, char* out);
void pf_format_list_real(double v, char* out);

/* ---- voxel analysis of the post-processor paraview.x (src/paraview.f90) ---
 * Per voxel (src/paraview.f90:189-244): phi_sq = sum_i phi_i^2; var_num = the
 * last variant with phi_i > 0.8 (0 if none); phi_3 = phi_3 (index 3 is fixed
 * in the reference); boundary = 1.0 where more than one phi_i > threshold;
 * grad_phi_3 = |grad phi_3| by central differences on interior cells, 0 on
 * the outer layer (:380-429).  Counts: boundary voxels, boundary voxels with
 * phi_var > threshold, and their ratio (0 without boundary voxels).  FP64 with
 * the reference's order of operations.  Needs var >= 3. */
typedef struct pf_voxel_counts {
  long long precipitate_voxels, boundary_voxels;
  double precipitate_fraction;
} pf_voxel_counts;
/* Host arrays of nx*ny*nz values in con(x,y,z) order; any may be NULL (not
 * computed / not copied back). */
typedef struct pf_analysis_out {
  double* phi_sq;
  int* var_num;
  double* phi_3;
  double* grad_phi_3;
  double* boundary;
  double* con; /* pf_analyze_run only: the run's c */
} pf_analysis_out;
/* Fields from host arrays (phi(var,x,y,z), con(x,y,z)) on cfg->device. */
int pf_analyze_fields(const pf_config* cfg, const double* phi_aos, const double* con, double threshold,
                      const pf_analysis_out* out, pf_voxel_counts* counts);
/* The resident fields of a run, with no host copy of the fields (out may be
 * NULL for the counts alone).  Leaves the run's state unchanged. */
int pf_analyze_run(pf_run* run, double threshold, const pf_analysis_out* out, pf_voxel_counts* counts);
/* An ASCII VTK file as paraview.f90:277-296 writes it: the fixed
 * STRUCTURED_POINTS header, then every value as one gfortran list-directed
 * record (REAL*8 or INTEGER*4 items), formatted on all host cores. */
int pf_write_vtk_real(const char* path, int nx, int ny, int nz, const double* v);
int pf_write_vtk_int(const char* path, int nx, int ny, int nz, const int* v);

/* Seeded starts (host only).  Draw order z, y, x (x fastest), per cell var phi
 * values then c, U(-a, a) = a (2 r - 1), r from ran_2 with idum = -(seed+1).
 * pf_ic_voronoi first draws n_grains points (Nx r, Ny r, Nz r); every cell
 * takes the nearest point (periodic minimum image, ties to the lower index)
 * and grain s sets variant (s mod var) to 1 before the noise is added. */
int pf_ic_noise(const pf_config* c, int seed, double amp_phi, double c0, double amp_c, double* phi_aos, double* con);
int pf_ic_voronoi(const pf_config* c, int seed, int n_grains, double amp_phi, double c0, double amp_c,
                  double* phi_aos, double* con);

#ifdef __cplusplus
}
#endif
#endif /* PFGPU_H */
