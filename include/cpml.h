/*
 * cpml.h -- C ABI of the GB300 staggered-grid velocity-stress elastic solver
 * with C-PML absorbing layers.
 *
 * This header is the drop-in boundary for the two reference programs
 *   seismic_CPML_2D_isotropic_second_order.f90       (2D P-SV, per-cell lambda/mu/rho)
 *   seismic_CPML_3D_isotropic_MPI_OpenMP.f90         (3D, homogeneous scalars)
 * Those programs have no callable API: their "interface" is the compile-time
 * parameter block (2D:138-218, 3D:124-218) and the output files they write.
 * Every entry point below names the reference lines whose behaviour it replaces.
 *
 * Conventions
 *   - Grid indices that cross this ABI are 1-based, as in the Fortran.
 *   - Host arrays are C order [k][j][i] (3D) or [j][i] (2D), i fastest; this
 *     is the same memory order as the Fortran arrays a(i,j,k), so a Fortran
 *     caller passes its arrays unchanged.
 *   - Seismograms are [nrec][nstep] doubles, the memory order of the Fortran
 *     sisvx(NSTEP,NREC).
 *   - Every function returns an int status (CPML_OK = 0, negative = error).
 *     Nothing aborts, exits or throws across this boundary.
 *   - The library owns device memory, streams and graphs per handle; it keeps
 *     no pointer to caller memory after a call returns. One handle = one CUDA
 *     stream; handles are independent; one handle is not thread-safe.
 */
#ifndef CPML_H
#define CPML_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CPML_OK              0
#define CPML_ERR_INVALID   (-1)  /* bad parameter or argument                  */
#define CPML_ERR_CFL       (-2)  /* Courant number > 1 (2D:513-516, 3D:712-717) */
#define CPML_ERR_OOM       (-3)  /* device allocation failed                    */
#define CPML_ERR_UNSTABLE  (-4)  /* max |v| > 1e25 or NaN (2D:716-726, 3D:1185-1195) */
#define CPML_ERR_TIMEOUT   (-5)  /* a bounded device-side wait gave up          */
#define CPML_ERR_CUDA      (-6)  /* a CUDA runtime call failed                  */
#define CPML_ERR_NOT_READY (-7)  /* results requested before they exist         */
#define CPML_ERR_IO        (-8)  /* host file output failed                     */
#define CPML_ERR_RANGE     (-9)  /* size beyond a documented maximum            */

/* ---- source time functions (2D:644-657, 3D:1055-1075) ------------------ */
#define CPML_STF_DGAUSSIAN 0     /* first derivative of a Gaussian (reference default, 2D:651) */
#define CPML_STF_GAUSSIAN  1     /* Gaussian (commented alternative, 2D:648)                   */
#define CPML_STF_RICKER    2     /* Ricker, second derivative (commented alternative, 2D:654)  */

/* ---- flags ------------------------------------------------------------- */
#define CPML_FLAG_ENERGY        0x1  /* record kinetic/potential energy every step (2D:694-713) */
#define CPML_FLAG_EP_PHYSICAL   0x2  /* 3D: use the textbook Ep (eps_zz*sigma_zz) instead of the
                                        reference's duplicated eps_yy*sigma_yy term (3D:1170-1171) */
#define CPML_FLAG_NO_STABILITY  0x4  /* skip the max|v| blow-up check at IT_DISPLAY cadence      */

/* ---- absorbing-layer schemes (cpml_params.scheme) ---------------------- */
#define CPML_SCHEME_CPML     0   /* convolutional PML, memory variables (the default) */
#define CPML_SCHEME_SPLIT    1   /* 2D only: classical split-field PML of Collino and
                                    Tsogka (seismic_PML_Collino_2D_isotropic.f90),
                                    homogeneous model, DELTAX = DELTAY, second order */

/* ---- step kernels (cpml_set_tuning) ----------------------------------- */
#define CPML_KERNEL_AUTO       0  /* 3D: fused one-sweep kernel; 2D: two-sweep         */
#define CPML_KERNEL_TWO_SWEEP  1  /* stress kernel + velocity kernel, in place          */
#define CPML_KERNEL_FUSED      2  /* 3D only: one kernel per step, two buffer sets, TMA  */
#define CPML_KERNEL_PERSISTENT 3  /* 2D only: the two sweeps of a whole chunk of steps in
                                     one cooperative launch, grid barriers between them;
                                     results bit-identical to CPML_KERNEL_TWO_SWEEP      */
#define CPML_KERNEL_CLUSTER    4  /* 2D second order only: the whole grid (fields, model,
                                     memory variables) in the shared memory of one
                                     thread-block cluster for a chunk of steps, halo rows
                                     exchanged through distributed shared memory; fields
                                     and seismograms bit-identical to TWO_SWEEP, energy
                                     summed per CTA (equal to rounding). CPML_ERR_INVALID
                                     when the grid does not fit on chip                 */

/* ---- fields (for cpml_get_field / cpml_get_plane) ---------------------- */
#define CPML_FIELD_VX  0
#define CPML_FIELD_VY  1
#define CPML_FIELD_VZ  2
#define CPML_FIELD_SXX 3
#define CPML_FIELD_SYY 4
#define CPML_FIELD_SZZ 5
#define CPML_FIELD_SXY 6
#define CPML_FIELD_SXZ 7
#define CPML_FIELD_SYZ 8

/*
 * Runtime copy of the reference's compile-time parameter block.
 * Field names follow the Fortran constants (2D:138-218, 3D:124-218).
 */
typedef struct cpml_params {
  int32_t ndim;          /* 2 or 3                                             */
  int32_t nx, ny, nz;    /* NX, NY, NZ (nz ignored in 2D)                      */
  int32_t nstep;         /* NSTEP: capacity of the seismogram/energy records  */
  int32_t npoints_pml;   /* NPOINTS_PML                                        */
  int32_t use_pml[6];    /* USE_PML_XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX (0/1)   */
  int32_t isource, jsource, ksource;  /* 1-based source grid point           */
  int32_t stf;           /* CPML_STF_*                                         */
  int32_t it_display;    /* IT_DISPLAY: cadence of the max|v| stability check */
  int32_t flags;         /* CPML_FLAG_*                                        */
  int32_t order;         /* spatial operator, 2D C-PML only: 0 or 2 = second
                            order (2D program); 4 = fourth order with the
                            27/24 staggered stencil (seismic_CPML_2D_isotropic_
                            fourth_order.f90:565-637)                         */
  int32_t scheme;        /* CPML_SCHEME_*                                      */
  int32_t reserved_i[2];
  double deltax, deltay, deltaz;  /* DELTAX, DELTAY, DELTAZ (m)               */
  double deltat;                  /* DELTAT (s)                               */
  double cp, cs, rho;    /* homogeneous model; cp also sets the PML d0 (2D:296) */
  double f0, t0, factor; /* source: dominant frequency, delay, amplitude       */
  double angle_force;    /* ANGLE_FORCE, degrees clockwise from +y (2D:176)   */
  double npower;         /* NPOWER (2D:213)                                    */
  double k_max_pml;      /* K_MAX_PML (2D:217)                                 */
  double alpha_max_pml;  /* ALPHA_MAX_PML (2D:218); <0 selects 2*pi*(f0/2)     */
  double rcoef;          /* Rcoef (2D:290)                                     */
  double reserved_d[4];
} cpml_params;

typedef struct cpml_handle cpml_handle;

/* Fill *p with the reference 2D program's parameter block (2D:138-218). */
int cpml_params_default_2d(cpml_params* p);
/* Fill *p with the parameter block of seismic_CPML_2D_isotropic_fourth_
   order.f90:132-190 (order 4, DELTAT halved and NSTEP and IT_DISPLAY doubled
   with respect to the second-order program). */
int cpml_params_default_2d_fourth(cpml_params* p);
/* Fill *p with the parameter block of seismic_PML_Collino_2D_isotropic.f90:
   96-141 (scheme CPML_SCHEME_SPLIT; h = DELTAX = DELTAY = 10 m). */
int cpml_params_default_2d_split(cpml_params* p);
/* Fill *p with the reference 3D program's parameter block (3D:124-218),
   single-domain semantics: source and receivers on global plane k = NZ/2. */
int cpml_params_default_3d(cpml_params* p);

/* Courant number cp*dt*sqrt(sum 1/d^2) (2D:513, 3D:712) for velocity cp_max;
   for CPML_SCHEME_SPLIT the split-field program's own one-dimensional number
   cp*dt/h (seismic_PML_Collino_2D_isotropic.f90:304), which lets time steps
   up to sqrt(2) beyond the 2D limit pass its check, as the program does. */
double cpml_courant(const cpml_params* p, double cp_max);

/* Nearest grid point to (x, y) metres by the reference's brute-force search:
   first minimum in i-fastest order wins (2D:486-509, 3D:683-706). 1-based out. */
int cpml_nearest_gridpoint(int nx, int ny, double deltax, double deltay,
                           double x, double y, int* i_out, int* j_out);

/* Build the 1-D C-PML profiles of one axis in FP64 on the host
   (2D:283-394 for x, 2D:396-465 for y, 3D:560-667 for z). Outputs are arrays
   of length n: d, K, alpha, a, b at grid points and at half points.
   Exposed so callers and tests can inspect what the device kernels use.
   Fourth order: the y axis's high-side origin is NY*DELTAY - thickness
   (2D4:401). CPML_SCHEME_SPLIT: d and d_half receive the split-field damping
   divided by two (seismic_PML_Collino_2D_isotropic.f90:180-250); K = 1,
   alpha = a = 0 and b = 1. */
int cpml_pml_profile(const cpml_params* p, int axis, int n,
                     double* d, double* K, double* alpha, double* a, double* b,
                     double* d_half, double* K_half, double* alpha_half,
                     double* a_half, double* b_half);

/* Create a solver: validates *p, checks the Courant number for the
   homogeneous cp (CPML_ERR_CFL, as 2D:516 stops), allocates device state,
   builds the C-PML tables in FP64 on the GPU and zeroes the wavefields
   (2D:522-544, 3D:720-756). Replaces the reference's set-up section. */
int cpml_create(const cpml_params* p, cpml_handle** out);

/* Per-cell model (host arrays, [k][j][i]): lambda, mu (Pa) and rho (kg/m^3),
   replacing the homogeneous fill of 2D:468-474. Any may be NULL to keep the
   homogeneous value. Re-checks the Courant number with max cp of the model. */
int cpml_set_model(cpml_handle* h, const float* lambda, const float* mu,
                   const float* rho);

/* Receivers as 1-based grid indices (2D:483-509, 3D:683-706 compute them from
   metres; use cpml_nearest_gridpoint for that). iz may be NULL in 2D and
   defaults to ksource in 3D (the reference records on the source plane). */
int cpml_set_receivers(cpml_handle* h, int nrec, const int* ix, const int* iy,
                       const int* iz);

/* Zero fields, memory variables, seismograms and energy; set it = 0 (the
   reference's initialisation, 2D:521-544, 3D:719-757). */
int cpml_reset(cpml_handle* h);

/* Advance nsteps time steps of the reference time loop (2D:550-735,
   3D:802-1245): stress + C-PML, velocity + C-PML, source, Dirichlet edges,
   receivers, energy, and the max|v| check every it_display steps.
   CPML_ERR_NOT_READY when the handle's last re-plan (cpml_set_model or
   cpml_set_tuning) failed part-way; a later successful one restores it. */
int cpml_run(cpml_handle* h, int nsteps);

/* Steps done so far and the last max|v| computed (2D:718, 3D:1185). */
/* Time steps done so far, and max |v| at the last display step (what the
   progress print-out shows, 2D:716-723, 3D:1183-1192). */
int cpml_status(cpml_handle* h, int* it, double* vmax);

/* Seismograms recorded so far, [nrec][nstep] doubles (sisvx/sisvy,
   2D:683-686, 3D:1124-1129). vz may be NULL; it is recorded for 3D only. */
int cpml_get_seismograms(cpml_handle* h, double* vx, double* vy, double* vz);

/* Kinetic and potential energy per step, nstep doubles each (2D:694-713,
   3D:1131-1180; the 3D reference writes only ek+ep). Either may be NULL. */
int cpml_get_energy(cpml_handle* h, double* ek, double* ep);

/* Copy one whole field to host FP32, [k][j][i] with nx*ny*nz values. No
   reference counterpart: the reference keeps its arrays inside the program. */
int cpml_get_field(cpml_handle* h, int field, float* out);

/* Copy one plane of a field: axis 0/1/2 = plane of constant i/j/k, index
   1-based. Output is row-major over the two remaining axes (slowest first).
   Used for the snapshots of 2D:729-732 and 3D:1236-1239 (k = NZ/2). */
int cpml_get_plane(cpml_handle* h, int field, int axis, int index, float* out);

/* Upload a whole field from host FP32 (tests and restarts). No reference
   counterpart. */
int cpml_set_field(cpml_handle* h, int field, const float* in);

/* Checkpoint / restart. The state a restart of the reference's time loop
   needs (3D:720-756, 2D:522-544 initialise it): the step counter it, the
   wavefields, every C-PML memory variable, and what has been recorded so far
   (seismograms, kinetic and potential energy, max|v| and the non-finite
   flags of steps 1..it). No reference counterpart: the reference programs
   run from it = 1 to NSTEP in one execution.
   cpml_state_size: bytes of a snapshot at the handle's current step.
   cpml_save_state: write the snapshot to caller-owned host memory (at least
     cpml_state_size bytes; CPML_ERR_RANGE if smaller).
   cpml_load_state: restore a snapshot into a handle created from the same
     parameter block, with the same per-cell model (cpml_set_model) and the
     same receivers (cpml_set_receivers) applied first; CPML_ERR_INVALID if
     the snapshot's grid, parameters, model or receivers differ. The step
     kernel may differ. Continuing the run gives bit for bit the results of
     the uninterrupted run. The format is this library's own (native byte
     order, a versioned header), not a portable file format. */
int cpml_state_size(cpml_handle* h, size_t* bytes);
int cpml_save_state(cpml_handle* h, void* buf, size_t bytes);
int cpml_load_state(cpml_handle* h, const void* buf, size_t bytes);

/* Bytes the hot path moves per time step by its compulsory count: every
   wavefield read and written once, per-cell model read once, each C-PML
   memory variable read and written once where its coefficient a is nonzero.
   For roofline figures; no reference counterpart. */
double cpml_algorithmic_bytes_per_step(cpml_handle* h);

/* Milliseconds of device time of the last cpml_run (CUDA events recorded on
   the handle's stream around it). No reference counterpart. */
int cpml_last_run_ms(cpml_handle* h, double* ms);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
   work or timing events against the solver's kernels. No reference
   counterpart: the reference has no device. */
int cpml_get_stream(cpml_handle* h, void** stream);

/* Select the step kernel (CPML_KERNEL_*; FUSED is 3D only, PERSISTENT and
   CLUSTER are 2D second order only: CPML_ERR_INVALID otherwise) and its
   launch shape: tile_y (rows of the 32-wide tile), zchunk (planes per CTA in
   the z sweep; each z range is cut into chunks of zchunk planes from its
   bottom, the shorter remainder last) and lookahead (planes the fused kernel's TMA loads run ahead
   of the plane being computed: 2, the only supported value). The shape only
   matters to the fused kernel. Supported (tile_y, lookahead): (8,2) (16,2).
   Single-shot kernels advance one time step per sweep: temporal blocking
   is the batched engine's (cpml_batch_set_tuning). Only on a fresh or reset
   handle. No reference counterpart: the reference's loop nests (3D:825-1052)
   have no tunables; the autotuner drives this. */
int cpml_set_tuning(cpml_handle* h, int kernel, int tile_y, int zchunk, int lookahead);
int cpml_get_tuning(cpml_handle* h, int* kernel, int* tile_y, int* zchunk, int* lookahead);
/* Kernels one time step launches with the current tuning, and kernels per
   chunk of steps (the FP64 reduction and the step counter); a chunk ends at
   it = 5 and every IT_DISPLAY steps. For launch accounting; no reference
   counterpart. */
int cpml_launches_per_step(cpml_handle* h, int* step_kernels, int* chunk_kernels);

/* Autotune the step kernel for this handle's grid: every candidate (3D: the
   one-sweep kernel with tile_y in {8,16} x zchunk in {16,24,32,40,48,64}; 2D:
   the persistent kernel and the on-chip cluster kernel where the grid fits;
   both: the two-sweep kernel) runs 2 untimed then trial_steps timed steps (CUDA events on the
   handle's stream); the fastest is applied. Results are cached per shape
   class (ndim, grid, per-cell model, NPML, PML faces) for the process and,
   when cache_path is not NULL, in that text file (one line per class). Leaves
   the handle reset. No reference counterpart. */
int cpml_autotune(cpml_handle* h, int trial_steps, const char* cache_path, int* kernel,
                  int* tile_y, int* zchunk, double* ms_per_step);

void cpml_destroy(cpml_handle* h);
const char* cpml_strerror(int status);

/* ---- batched 2D shots ---------------------------------------------------
   Many independent runs of the 2D program (2D:550-735), each with its own
   grid, model, source, receivers, DELTAT and NSTEP, advanced together in one
   persistent cooperative kernel launch captured in a CUDA graph. A shot's
   seismograms and fields are bit-identical to a single-shot handle running
   the same parameters (same per-cell arithmetic). No counterpart in the
   reference, which runs one shot per program execution; energy is not
   recorded by the batched engine. Shots run the second-order C-PML program:
   a shot with order 4 or the split-field scheme is CPML_ERR_INVALID. */
typedef struct cpml_batch cpml_batch;
int cpml_batch_create(int nshots, const cpml_params* params, cpml_batch** out);
int cpml_batch_set_model(cpml_batch* b, int shot, const float* lambda, const float* mu,
                         const float* rho);
int cpml_batch_set_receivers(cpml_batch* b, int shot, int nrec, const int* ix, const int* iy);
/* Zero every shot and run each to its own NSTEP. */
int cpml_batch_run(cpml_batch* b);
int cpml_batch_get_seismograms(cpml_batch* b, int shot, double* vx, double* vy);
int cpml_batch_get_field(cpml_batch* b, int shot, int field, float* out);
int cpml_batch_last_run_ms(cpml_batch* b, double* ms);
/* Bound, in SM clock cycles, of one wait at the engine's grid barrier
   (0 restores the default, about 2 s). A wait that runs out makes
   cpml_batch_run return CPML_ERR_TIMEOUT with every CTA of the launch
   returned; the next run starts clean. For tests of that path. */
int cpml_batch_set_wait_limit(cpml_batch* b, long long cycles);
/* Temporal blocking of the batched engine: depth = time steps a tile
   advances in shared memory per HBM round trip and per grid barrier, tile_y
   = rows of its 32-wide tiles. Supported (depth, tile_y): (1, 8) the
   two-barrier-per-step engine, (2, 8), (2, 16), (3, 16). Results are
   bit-identical for every choice. Depth > 1 allocates a second buffer set
   per shot (fields and memory variables). No reference counterpart. */
int cpml_batch_set_tuning(cpml_batch* b, int depth, int tile_y);
int cpml_batch_get_tuning(cpml_batch* b, int* depth, int* tile_y);
/* Time the first trial_steps steps of the batch under every supported
   (depth, tile_y) (CUDA events around the launch) and keep the fastest;
   the batch is left ready for cpml_batch_run. No reference counterpart. */
int cpml_batch_autotune(cpml_batch* b, int trial_steps, int* depth, int* tile_y, double* ms_per_step);
void cpml_batch_destroy(cpml_batch* b);

/* Kinetic and potential energy (the 3D program's formulas, 3D:1131-1180) of
   nine caller-owned FP32 device wavefields, allocating no device memory.
   No counterpart in the reference: it serves callers that cannot allocate
   device memory mid-run (a host that owns its fields through its own pool or
   a fixed memory budget, where cudaMalloc would synchronise or fail).
     fields: 9 device pointers vx vy vz sxx syy szz sxy sxz syz, each
             [nz][ny][pitch] floats (pitch >= nx, in floats);
     npml:   interior = [npml, n - npml) on every axis (CPML_ERR_INVALID
             unless 2*npml < nx, ny and nz);
     lam/mu/rho: homogeneous model, used when the three *_cell device arrays
             (same layout as the fields) are NULL;
     flags:  CPML_FLAG_EP_PHYSICAL selects the textbook Ep;
     out:    device pointer to 2 doubles (Ek, Ep), written on `stream`.
   Scratch is a static device array of per-plane sums for at most 8192 planes
   (nz > 8192 returns CPML_ERR_RANGE). Its address is looked up on a device's
   first call, so make that call before any stream capture; the address is
   kept for the life of the process, so a device or context reset between
   calls is not supported. All calls share that array: calls that overlap
   on the GPU race, so order them. */
int cpml_energy3d_noalloc(const float* const* fields, int nx, int ny, int nz, int pitch,
                          int npml, double lam, double mu, double rho,
                          const float* lam_cell, const float* mu_cell,
                          const float* rho_cell, int flags, double* out, void* stream);

/* ---- learned-surrogate network kernels -----------------------------------
   No counterpart in the reference. The building blocks of a small
   convolutional network that predicts 2D receiver seismograms from a
   velocity model and a source position; shots it predicts poorly are re-run
   by the FD solver. All pointers are device pointers; "bf16" buffers hold
   IEEE bfloat16 values; every call is asynchronous on `stream`.

   cpml_nn_gemm: C[M,N] = alpha * op(A)[M,K] op(B)[K,N] on BF16 tensor cores
   with FP32 accumulation. ta = 0: A is [M][lda]; ta = 1: A is [K][lda].
   tb = 0: B is [K][ldb]; tb = 1: B is [N][ldb]. Then + bias[n] (bias may be
   NULL), + the old Cf if accum, ReLU if relu, and stores to Cf (FP32) and/or Cb
   (bf16), row stride ldc. splits > 1 splits K; the partial sums go to `work`
   (>= splits*M*N floats) and are added in split order. */
int cpml_nn_gemm(int M, int N, int K, const void* A, int lda, int ta, const void* B, int ldb, int tb,
                 float* Cf, void* Cb, int ldc, const float* bias, int relu, int accum, float alpha,
                 int splits, float* work, long long work_elems, void* stream);
/* The same contract as cpml_nn_gemm on the 5th-generation tensor cores
   (tcgen05.mma, accumulator in tensor memory; 128-row output tiles 32, 64 or
   128 columns wide, the narrowest that covers N). */
int cpml_nn_gemm_tc(int M, int N, int K, const void* A, int lda, int ta, const void* B, int ldb, int tb,
                    float* Cf, void* Cb, int ldc, const float* bias, int relu, int accum, float alpha,
                    int splits, float* work, long long work_elems, void* stream);
/* *err = whether a bounded tensor-core wait gave up since the last call
   (1) or not (0); resets the flag. Synchronous. */
int cpml_nn_error(int* err);
/* 3x3 stride-2 pad-1 patches of an NHWC bf16 [B][H][W][C] activation:
   out [B*Ho*Wo][9*C] bf16, Ho = (H+1)/2, column (ky*3+kx)*C + c. */
int cpml_nn_im2col(const void* in, void* out, int B, int H, int W, int C, void* stream);
/* Adjoint of cpml_nn_im2col on FP32 data: out [B][H][W][C] (overwritten). */
int cpml_nn_col2im(const float* col, float* out, int B, int H, int W, int C, void* stream);
/* dx = dy where y > 0, else 0; to bf16 and/or FP32 (either may be NULL). */
int cpml_nn_relu_bwd(const float* dy, const float* y, void* dx_bf16, float* dx_f32, long long n,
                     void* stream);
/* dst[b][r][:] = src[b][r + shift[b]][:] (L values per row) where
   0 <= r + shift[b] < rows_src, else 0; dst has rows_dst rows per shot, to
   FP32 and/or bf16. shift is a device int array of B entries. */
int cpml_nn_shift_rows(const float* src, const int* shift, float* dst_f32, void* dst_bf16, int B,
                       int rows_src, int rows_dst, int L, void* stream);
int cpml_nn_cast(const float* x, void* y_bf16, long long n, void* stream);
/* out[n] (+)= sum over m of x[m][n]; work >= ceil(M/256)*N floats. */
int cpml_nn_colsum(const float* x, float* out, int M, int N, int accum, float* work,
                   long long work_elems, void* stream);
/* Per shot b of B rows of L values: loss[b] = ||pred-target||^2 / ||target||^2
   and, if grad != NULL, grad = d(mean_b loss[b]) / d pred. */
int cpml_nn_rel_l2(const float* pred, const float* target, float* grad, float* loss, int B, int L,
                   void* stream);
/* dh[b] = d/dh_b of weight * mean_b (h[b*ldh] - log loss[b])^2. */
int cpml_nn_head_grad(const float* h, int ldh, const float* loss, float* dh, int B, float weight,
                      void* stream);
/* One Adam step (bias-corrected with `step`, 1-based; L2 weight decay wd) on
   n FP32 master weights w, refreshing their bf16 copy wb (may be NULL). */
int cpml_nn_adam(float* w, void* wb, const float* g, float* m, float* v, long long n, float lr,
                 float beta1, float beta2, float eps, int step, float wd, void* stream);

/* ---- reference output files (2D:738-808, 820-999; 3D:1247-1364) -------- */

/* Vx_file_NNN.dat / Vy_file_NNN.dat (/ Vz_file_NNN.dat if vz != NULL), one
   "t v" line per step in Fortran list-directed REAL(4) style (2D:820-854). */
int cpml_write_seismograms(const char* dir, const double* vx, const double* vy,
                           const double* vz, int nt, int nrec, double deltat);

/* Binary receiver output for large receiver sets: seisVx.su, seisVy.su (and
   seisVz.su if vz != NULL), the Seismic Unix layout the reference's
   seismic_ADEPML_2D_elastic_RK4_eighth_order.f90:985-1004 writes with
   access='stream': per receiver a 240-byte header of 120 native-order int16
   words, all zero except word 58 = nt and word 59 = trunc(deltat*1e6)
   (microseconds), then nt REAL(4) samples. vx/vy/vz are [nrec][nt].
   CPML_ERR_RANGE when nt or the interval in microseconds exceeds 32767. */
int cpml_write_seismograms_su(const char* dir, const double* vx, const double* vy,
                              const double* vz, int nt, int nrec, double deltat);

/* energy.dat: 2D writes t, Ek, Ep, Ek+Ep (2D:741-746); 3D writes t, Ek+Ep
   (3D:1253-1257). ncol selects 4 or 2. */
int cpml_write_energy(const char* dir, const double* ek, const double* ep,
                      int nt, double deltat, int ncol);

/* imageNNNNNN_Vx.pnm / _Vy.pnm colour snapshot (2D:861-999). data is one
   [ny][nx] plane; field_number 1 = Vx, 2 = Vy. */
int cpml_write_pnm(const char* dir, const float* data, int nx, int ny, int it,
                   int isource, int jsource, const int* ix_rec,
                   const int* iy_rec, int nrec, int npoints_pml,
                   const int* use_pml4, int field_number);

#ifdef __cplusplus
}
#endif
#endif /* CPML_H */
