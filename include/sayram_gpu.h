/*
 * sayram_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of Sayram-2D's per-time-step hot
 * path: the PPFV (Gao-Wu) assembly of nonlinear two-point-flux coefficients with cross
 * diffusion, the loss term folded into the matrix, and the implicit linear solve.
 *
 * Plain C types only (no CUDA or torch types), so any FFI (ctypes, cgo, JNI, a C++ wrapper) can
 * bind it.  Every function returns a status code (SAYRAM_OK = 0) and never throws; the message
 * of the last failure on the calling thread is available from sayram_last_error().
 *
 * Reference interface each group replaces (Sayram-2D, paths relative to its repository):
 *   sayram_create / sayram_update / sayram_t / sayram_get_f / sayram_destroy
 *       -> class Solver (source/Solver.h:18-26): Solver(const Mesh&, Equation*) [Solver.cc:14-34],
 *          void update() [Solver.cc:270-290], double t() const [Solver.h:23],
 *          const Xtensor2d& f() const [Solver.h:24].
 *   sayram_problem
 *       -> what Solver reads from Mesh (source/Mesh.h:38-63: edges, dt) and from Equation
 *          (source/Equation.h:44-65: G, Dxx, Dxy, Dyy, inv_tau, init_f, bc_type,
 *          dirichlet_vertex_value), evaluated into arrays.
 *   sayram_set_dirichlet / sayram_set_coeffs
 *       -> the per-step re-reads after eq.update(t) (Solver.cc:286-289: update_Lambda and
 *          fill_vertex_from_bcs), for cases whose coefficients or boundary values change.
 *   sayram_dtable / sayram_set_dtable / sayram_batch_set_dtable
 *       -> Albert_Young(_LC)::constructD (source/Cases/Albert_Young.cc:112-134) with locate
 *          (Albert_Young.cc:94-110), calWeight and interp2D (source/utils.h:24-58): the D fields
 *          interpolated from the case's HDF5 D table (Albert_Young_IO.cc:17-36), on the device.
 *   sayram_batch_*   -> no counterpart (many independent Solver instances advanced together).
 *   sayram_server_*  -> no counterpart (continuous-batching service of solve requests).
 *
 * Array layouts follow the reference: per-cell fields are (nx, ny) alpha-major, element (i, j)
 * at i*ny + j (xtensor row-major, as Equation::G_ etc.).  Dirichlet vertex values of sides
 * XMIN/XMAX are indexed by j = 0..ny, of YMIN/YMAX by i = 0..nx (Solver.cc:398-419).
 */
#ifndef SAYRAM_GPU_H
#define SAYRAM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define SAYRAM_OK 0
#define SAYRAM_ERR_ARG 1           /* invalid argument (bad grid, missing Dirichlet values, ...) */
#define SAYRAM_ERR_OOM 2           /* device or host allocation failed */
#define SAYRAM_ERR_NOT_CONVERGED 3 /* a step ended above the residual target (state still advanced) */
#define SAYRAM_ERR_NEGATIVE 4      /* a negative cell survived the positivity polish */
#define SAYRAM_ERR_TIMEOUT 5       /* a bounded device wait ran out */
#define SAYRAM_ERR_CUDA 6          /* CUDA runtime error (no device, launch failure, ...) */
#define SAYRAM_ERR_BUDGET 7        /* request does not fit the serving HBM budget */
#define SAYRAM_ERR_STATE 8         /* call not valid in the object's current state */
#define SAYRAM_ERR_IO 9            /* file could not be created or written */

/* ---- boundary ids and types (source/BCTypes.h:13-16) ------------------------------------ */
#define SAYRAM_XMIN 0
#define SAYRAM_XMAX 1
#define SAYRAM_YMIN 2
#define SAYRAM_YMAX 3
#define SAYRAM_DIRICHLET 0
#define SAYRAM_ZEROFLUX 1

/* ---- precision modes --------------------------------------------------------------------- */
#define SAYRAM_FP64 0        /* FP64 everywhere (the plain drop-in) */
#define SAYRAM_FP32_REFINE 1 /* FP32 matrix/Krylov, FP64 residual + refinement + checks */
#define SAYRAM_FP32_REFINE_DW 2 /* FP32 matrix/Krylov; the residual, refinement, assembly and
                                   checks in double-word arithmetic (pairs of FP32, ~48-bit
                                   significand) on the FP32 pipes -- GB300's FP64 rate is 1/69 of
                                   its FP32 rate */

/* One instance: grid, time step, coefficients, initial state and boundary conditions. All
 * arrays are read during the call that receives the struct and are not retained. */
typedef struct sayram_problem {
  int nx, ny;               /* cells in alpha0 (x) and log E (y) */
  const double* x_edges;    /* nx+1, strictly increasing (Grid2D.h:44-67) */
  const double* y_edges;    /* ny+1, strictly increasing */
  double dt;                /* time step (Mesh::dt, Mesh.h:55) */
  int bc[4];                /* SAYRAM_DIRICHLET or SAYRAM_ZEROFLUX for XMIN, XMAX, YMIN, YMAX */
  const double* G;          /* (nx, ny) alpha-major: Jacobian factor */
  const double* Dxx;        /* diffusion tensor components */
  const double* Dxy;
  const double* Dyy;
  const double* inv_tau;    /* loss rate 1/tau (0 = no loss) */
  const double* f0;         /* initial state (Equation::init_f at cell centres) */
  const double* dirichlet[4]; /* vertex values per side; NULL for zero-flux sides */
} sayram_problem;

typedef struct sayram_options {
  int precision;    /* SAYRAM_FP64 (default), SAYRAM_FP32_REFINE or SAYRAM_FP32_REFINE_DW */
  double tol;       /* target ||R - M f|| / ||R|| in the Jacobi-scaled system (FP64 residual);
                       default 1e-12 (FP64) / 1e-11 (FP32_REFINE, FP32_REFINE_DW) */
  double inner_tol; /* residual reduction asked of each inner Krylov solve; default 0 (FP64:
                       solve to tol at once) / 1e-4 (FP32 modes) */
  int max_iters;    /* inner BiCGSTAB iterations per solve; default 500 */
  int max_refine;   /* FP64 residual evaluations (outer refinements) per step; default 6 */
  int device;       /* CUDA device ordinal; default 0 */
  int use_graph;    /* 1 (default): each step runs as one CUDA graph with device-side loops */
  int precond;      /* preconditioner of the inner Krylov solve, applied on the left:
                       SAYRAM_PRECOND_JACOBI (0): the unit-diagonal (Jacobi) scaling only;
                       SAYRAM_PRECOND_ALPHA_LINE (1, default): also the alpha-line blocks -- the
                       tridiagonal of the west/east couplings over each aligned 4-cell piece of a
                       row, solved exactly (block Jacobi with 4-cell alpha-line blocks). A caller
                       that zero-fills the struct instead of calling sayram_default_options gets
                       Jacobi. The converged answer does not depend on it. */
} sayram_options;

enum { SAYRAM_PRECOND_JACOBI = 0, SAYRAM_PRECOND_ALPHA_LINE = 1 };

typedef struct sayram_stats {
  long long steps;        /* steps taken since creation */
  double t;               /* simulated time = steps * dt (Solver::t, Solver.h:23) */
  int status;             /* status of the last step: SAYRAM_OK / NOT_CONVERGED / NEGATIVE */
  int refinements;        /* FP64 residual evaluations in the last step */
  int iterations;         /* inner Krylov iterations in the last step */
  double rel_residual;    /* final FP64 ||R - M f||/||R|| of the last step (scaled system) */
  double min_f;           /* minimum cell value after the positivity polish */
  long long clamped;      /* cells the polish lifted from a negative Krylov value */
  double mass_drift;      /* |1^T M f - 1^T R| / 1^T R after the last step */
  long long total_iterations;  /* inner Krylov iterations since creation */
  long long total_refinements; /* FP64 residual evaluations since creation */
} sayram_stats;

/* ---- library -------------------------------------------------------------------------- */
const char* sayram_last_error(void); /* message of the last failure on this thread ("" if none) */
const char* sayram_version(void);
void sayram_default_options(sayram_options* opt);
/* Pinned host memory for fast host<->device copies (cudaMallocHost); NULL on failure. */
void* sayram_host_alloc(size_t bytes);
void sayram_host_free(void* p);

/* ---- single instance: the drop-in for class Solver -------------------------------------- */
typedef struct sayram_batch_s* sayram_solver;

/* Solver::Solver(const Mesh&, Equation*): copies the problem to the device. */
int sayram_create(const sayram_problem* p, const sayram_options* opt, sayram_solver* out);
/* Solver::update(): one backward-Euler step (assembly from the current f, solve, polish). */
int sayram_update(sayram_solver s);
/* nsteps calls of update() without returning to the host in between. */
int sayram_step(sayram_solver s, int nsteps);
/* Solver::t() */
double sayram_t(sayram_solver s);
/* Solver::f(): copies f (alpha-major, nx*ny doubles) to the host. */
int sayram_get_f(sayram_solver s, double* f_out);
/* Replaces f (alpha-major). */
int sayram_set_f(sayram_solver s, const double* f);
/* New Dirichlet vertex values for one side (n = ny+1 for XMIN/XMAX, nx+1 for YMIN/YMAX). */
int sayram_set_dirichlet(sayram_solver s, int side, const double* v, int n);
/* New G, D and 1/tau fields (alpha-major); all five are required. */
int sayram_set_coeffs(sayram_solver s, const double* G, const double* Dxx, const double* Dxy,
                      const double* Dyy, const double* inv_tau);
int sayram_get_stats(sayram_solver s, sayram_stats* out);
void sayram_destroy(sayram_solver s);

/* A diffusion-coefficient table as the Albert_Young cases read it from D/<dID>.h5
 * (Albert_Young_IO::read_D): the datasets /alpha0 (degrees), /E, /Daa, /Dap, /Dpp. */
typedef struct sayram_dtable {
  int n_alpha, n_energy;          /* nodes along alpha0 and E, both >= 2 */
  const double* alpha0_deg;       /* n_alpha pitch angles in degrees (/alpha0) */
  const double* energy;           /* n_energy energies (/E), > 0 */
  const double *Daa, *Dap, *Dpp;  /* n_alpha x n_energy, row-major (alpha0-major), as stored */
} sayram_dtable;
/* Replaces Dxx, Dxy, Dyy by the table interpolated at the cell centres, on the device, as the
 * reference's constructD does: positions from the axes' end points (uniform in alpha0 and in
 * log E assumed), bilinear weights, the last node beyond the table's upper ends, then
 * Dxx = Daa k / p^2, Dxy = Dap k (dlogE/dp) / p, Dyy = Dpp k (dlogE/dp)^2 with k = gME^2 gC^2 *
 * 86400 and p = e2p(E) at the cell's E. A centre below the table's first node takes the first
 * node (the reference's own calWeight branch for that case; its size_t conversion there is
 * undefined). G, 1/tau, f and the boundary values stay. Only the table crosses to the device. */
int sayram_set_dtable(sayram_solver s, const sayram_dtable* t);

/* ---- batches: many independent instances advanced by the same launches ------------------- */
typedef struct sayram_batch_s* sayram_batch;

/* A batch holds fewer than 2^31 - 1 padded cells (SAYRAM_ERR_ARG otherwise): the assembly
 * indexes cells with 32-bit integers, and that many cells would need ~330 GB of device memory. */
int sayram_batch_create(const sayram_problem* probs, int n, const sayram_options* opt,
                        sayram_batch* out);
int sayram_batch_size(sayram_batch b);
/* Advances every instance by nsteps. Returns NOT_CONVERGED / NEGATIVE if any instance's last
 * step did (per-instance detail in sayram_batch_stats). */
int sayram_batch_step(sayram_batch b, int nsteps);
/* The end-to-end form: if f_in is not NULL it first replaces every instance's f from the packed
 * host array (instances concatenated, each alpha-major), then steps, then, if f_out is not
 * NULL, writes every instance's f back the same way. Pinned buffers (sayram_host_alloc) copy
 * fastest. The first guess of each step's solve is extrapolated from the last few states; an
 * instance whose f_in differs from the state it holds restarts that history, one given back its
 * own f_out unchanged keeps it (results never depend on the guess, only the iteration count).
 * The copies overlap the computation: runs of instances are copied in while the first step
 * assembles the runs already on the device, and copied out while the last step's positivity
 * polish finishes the later runs; the result is bit for bit that of sayram_batch_step. */
int sayram_batch_step_host(sayram_batch b, int nsteps, const double* f_in, double* f_out);
int sayram_batch_get_f(sayram_batch b, int idx, double* f_out);
int sayram_batch_set_f(sayram_batch b, int idx, const double* f);
int sayram_batch_set_dirichlet(sayram_batch b, int idx, int side, const double* v, int n);
int sayram_batch_set_coeffs(sayram_batch b, int idx, const double* G, const double* Dxx,
                            const double* Dxy, const double* Dyy, const double* inv_tau);
/* As sayram_set_dtable for instance idx, or for every instance when idx < 0 (one launch). */
int sayram_batch_set_dtable(sayram_batch b, int idx, const sayram_dtable* t);
int sayram_batch_stats(sayram_batch b, int idx, sayram_stats* out);
/* Assembles instance idx's linear system from its current f (without stepping) and returns it
 * in the reference's unscaled form M f = R (the M_ and R_ members of Solver, Solver.h:37-41),
 * system order K = j*nx + i: M5 holds five diagonals of nx*ny each -- M(K,K), M(K,K-1),
 * M(K,K+1), M(K,K-nx), M(K,K+nx) (0 where the neighbour does not exist) -- and R nx*ny. */
int sayram_batch_export_system(sayram_batch b, int idx, double* M5, double* R);
/* Total device bytes held by the batch. */
size_t sayram_batch_device_bytes(sayram_batch b);
/* The CUDA stream the batch launches on (a cudaStream_t, as void*), for event timing. */
void* sayram_batch_stream(sayram_batch b);
/* CUDA events on the batch's stream: record event slot (0..7); elapsed time between two recorded
 * slots (waits for the later one). */
int sayram_batch_record_event(sayram_batch b, int slot);
int sayram_batch_elapsed_ms(sayram_batch b, int slot0, int slot1, double* ms);
/* Per-kernel timing: when enabled, every launch is bracketed by CUDA events on the batch's
 * stream (steps then run without graphs). sayram_batch_kernel_times fills up to cap entries of
 * names/total milliseconds/launch counts and returns the number of entries: one per kernel, plus
 * "krylov_tail10" and "krylov_rest", the time of whole BiCGSTAB iterations (their three kernels)
 * in which fewer than 10 % / at least 10 % of the enabled instances were still iterating. */
int sayram_batch_enable_timing(sayram_batch b, int enable);
int sayram_batch_kernel_times(sayram_batch b, const char** names, double* total_ms,
                              long long* launches, int cap);
/* Autotuner: times `steps` steps of each launch shape -- cells per block iteration (1024, 2048,
 * 4096) x blocks per SM in the grid (8, 16, 32, 64) -- on this batch's own instances and keeps the
 * fastest. The instances' state is restored afterwards, so tuning does not advance the
 * simulation. Writes the choice if the pointers are not NULL. */
int sayram_batch_autotune(sayram_batch b, int steps, int* chunk_out, int* blocks_per_sm_out);
/* The refinement loop of a step runs as one cooperative kernel (grid-wide barriers between its
 * passes) when every chunk of the batch gets a block in one wave of co-resident blocks -- a
 * single large instance or a few -- and as the graph's loops of separate kernels otherwise.
 * on = 0 always uses the separate kernels (the results are the same bit for bit). Default: 1. */
int sayram_batch_set_coop(sayram_batch b, int on);
/* Sets the launch shape directly (chunk 1024, 2048 or 4096 cells; 1..64 blocks per SM), or reads
 * it back. The default is chosen from the batch size; results do not depend on it beyond the
 * order of the reductions. */
int sayram_batch_set_launch_shape(sayram_batch b, int chunk, int blocks_per_sm);
int sayram_batch_get_launch_shape(sayram_batch b, int* chunk, int* blocks_per_sm);
/* The timings of the last autotune: up to cap (chunk, blocks per SM, ms per step) entries;
 * returns the number of candidates measured. */
int sayram_batch_tuning_log(sayram_batch b, int* chunks, int* blocks_per_sm, double* ms_per_step, int cap);
/* Kernel launches issued by this batch since creation (counted on the device). */
long long sayram_batch_launches(sayram_batch b);
void sayram_batch_destroy(sayram_batch b);

/* ---- serving: continuous batching of solve requests -------------------------------------
 * No counterpart in the reference. A server owns a device arena sized by an HBM budget. Requests
 * (a problem plus a step count) are queued by sayram_server_submit; every sayram_server_tick
 *   1. admits waiting requests in arrival order while a slot and a contiguous region of the arena
 *      are free (a request that does not fit waits; up to 8 later requests may pass it),
 *   2. advances every resident instance by one backward-Euler step, all in the same launches,
 *   3. copies the state of instances that reached their step count back to the host and frees
 *      their memory, so that the next tick can admit more.
 * Each instance's f, coefficients and matrix stay on the device from admission to completion.
 * Results are collected with sayram_server_poll. Latency = completion - submission (steady clock). */
typedef struct sayram_server_s* sayram_server;

typedef struct sayram_server_config {
  double hbm_budget_bytes; /* device bytes the server may use (arena + tables + solver state) */
  int max_slots;           /* instances resident at once, per lane (default 4096) */
  int max_side;            /* largest nx or ny accepted (default 1024) */
  /* Lanes (0 or 1: one). With 2, requests with max(nx, ny) <= lane_split_side (default 128) run
   * in a lane of their own -- its own stream, arena (lane_small_fraction of the budget, default
   * 0.25) and work lists -- so that their steps do not wait for the Krylov iterations of large
   * grids; each tick collects whichever lanes have finished a step and relaunches the idle ones. */
  int lanes;
  int lane_split_side;
  double lane_small_fraction;
  /* Longest a tick waits on the host for a lane's step to finish (seconds; <= 0: 600). A tick
   * that gives up returns SAYRAM_ERR_TIMEOUT and leaves the step in flight; a later tick waits
   * for it again and collects it. */
  double wait_seconds;
} sayram_server_config;

typedef struct sayram_server_info {
  long long submitted, admitted, completed, waiting, resident;
  long long ticks;              /* steps run, summed over the lanes */
  long long instance_steps;     /* steps executed, summed over instances */
  double device_bytes;          /* bytes held by the server */
  double arena_cells, arena_cells_used;
  double busy_seconds;          /* wall time spent inside ticks that ran a step */
  double admit_seconds;         /* of which: admitting requests (copies + set-up) */
  double lists_seconds;         /*           rebuilding the work lists */
  double step_seconds;          /*           launching the step and waiting for it */
  double collect_seconds;       /*           copying finished results out */
} sayram_server_info;

int sayram_server_create(const sayram_server_config* cfg, const sayram_options* opt, sayram_server* out);
/* Copies the problem (arrays are not retained) and queues it for nsteps steps. SAYRAM_ERR_BUDGET
 * if the request could never fit the server (grid larger than max_side or than the arena). */
int sayram_server_submit(sayram_server s, const sayram_problem* p, int nsteps, long long* id_out);
/* One scheduling round: every idle lane admits waiting requests and launches one step of its
 * resident instances; the call returns when at least one lane's step has finished, after copying
 * out the instances of the finished lanes that reached their step count. With one lane: admission,
 * one step of every resident instance, completions. */
int sayram_server_tick(sayram_server s, int* n_completed);
/* SAYRAM_OK and the result (f alpha-major, stats, submit/done times in seconds of the steady
 * clock) when request id has completed -- the result is then released; SAYRAM_ERR_STATE if not
 * yet. Any output pointer may be NULL. */
int sayram_server_poll(sayram_server s, long long id, double* f_out, sayram_stats* st, double* t_submit,
                       double* t_done);
int sayram_server_info_get(sayram_server s, sayram_server_info* out);
/* Ids of completed requests not yet polled (up to cap); returns how many were written. */
int sayram_server_completed_ids(sayram_server s, long long* ids, int cap);
void sayram_server_destroy(sayram_server s);

/* ---- stepping without allocating -------------------------------------------------------
 * sayram_step_noalloc: nsteps FP64 backward-Euler steps of ONE instance that allocate no memory.
 * No counterpart in the reference. It is for callers that cannot call cudaMalloc: programs whose
 * own memory manager owns the GPU's memory (for example a larger model that embeds this step and
 * reserves the device through its own pool), and programs that must not allocate once running
 * (a memory budget fixed at start, where an allocation failure mid-run is not acceptable).
 *
 * Every array pointer in *p (edges, G, Dxx, Dxy, Dyy, inv_tau, Dirichlet values) and f_in/f_out
 * is a DEVICE pointer, with the same layouts as for sayram_create; p->f0 is ignored and the state
 * comes from f_in (alpha-major). f_out may equal f_in. stream is a cudaStream_t (NULL = legacy
 * default stream); the call returns once that stream has finished the work. opt may be NULL and
 * must select SAYRAM_FP64. stats (may be NULL) receives this call's statistics.
 *
 * Working memory is one fixed device array of 16,973,824 bytes defined in this library; every
 * GPU that loads the library holds it until the process exits. A grid fits when
 * round_up((ny+2) * round_up(nx,4), 32) + 64 <= 73728 cells and nx, ny <= 4096 (256 x 256
 * fits); larger grids return SAYRAM_ERR_ARG with a message saying so.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress) and
 * keeps it for later calls; make that first call before any stream capture begins. The kept
 * address does not survive cudaDeviceReset: calls after a reset are not supported. Every call
 * waits for its stream between launches (it reads the loops' control words back to the host).
 * All calls share the array: each call clears it at its start and the array keeps the last
 * call's contents afterwards. Calls that overlap on the GPU (several host threads or streams at
 * once) race on it and must be serialized by the caller. */
int sayram_step_noalloc(const sayram_problem* p, const sayram_options* opt, int nsteps,
                        const double* f_in, double* f_out, void* stream, sayram_stats* stats);

/* Bytes of device memory an instance of nx*ny cells needs (admission control). */
size_t sayram_instance_bytes(int nx, int ny, int precision);

#ifdef __cplusplus
}
#endif

#endif /* SAYRAM_GPU_H */
