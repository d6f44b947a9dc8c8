/*
 * miniaero_gpu.h -- C ABI of libminiaero_gpu.so, the GB300 (sm_103a)
 * implementation of miniAero's explicit RK4 residual path.
 *
 * Plain C types only: pointers, sizes, status codes. The library owns all
 * device memory; host pointers passed in are borrowed for the duration of the
 * call. Every function returns ma_status (0 = MA_OK); on failure
 * ma_last_error() returns a message for the calling thread. No C++ exception
 * crosses this boundary.
 *
 * Each entry point names the reference interface it replaces
 * (kokkos/<file>:<line> in Mantevo miniAero).
 */
#ifndef MINIAERO_GPU_H_
#define MINIAERO_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MA_ABI_VERSION 1

typedef enum {
  MA_OK = 0,
  MA_EINVAL = 1,     /* bad argument or option */
  MA_ENOMEM = 2,     /* host or device allocation failed */
  MA_ECUDA = 3,      /* CUDA runtime error (no device, launch failure, ...) */
  MA_EBUDGET = 4,    /* request does not fit the device-memory budget */
  MA_ETIMEDOUT = 5,  /* bounded wait expired */
  MA_ENUMERIC = 6,   /* non-finite or non-physical state detected */
  MA_ESTATE = 7,     /* call not valid in the object's current state */
  MA_EIO = 8,        /* file could not be read or written */
  MA_ENOTFOUND = 9   /* unknown id */
} ma_status;

enum { MA_BC_EXTRAPOLATE = 0, MA_BC_TANGENT = 1, MA_BC_INFLOW = 2, MA_BC_NOSLIP = 3 };
enum { MA_LIMITER_VENKAT = 0, MA_LIMITER_VANALBADA = 1 };
enum { MA_VISC_SUTHERLAND = 0, MA_VISC_CONSTANT = 1 };
/* MA_PREC_FP64: the reference's serial arithmetic, bit for bit.
 * MA_PREC_MIXED: FP32 flux, gradient and limiter; FP64 residual sum and RK4
 * update (relative L2 density error <= 1e-5 against FP64).
 * MA_PREC_FP64_FMA: the FP64 kernels with a*b+c fused where the compiler
 * contracts it (as an aarch64 build of the reference with default flags
 * does); same summation orders, round-off-level differences from the
 * reference's bits that grow with the flow (opt-in; within 1e-12 on the
 * benchmark meshes after their configured steps, 7e-9 after the reference's
 * 400-step flat plate, where its own serial and threaded builds differ as
 * much). */
enum { MA_PREC_FP64 = 0, MA_PREC_MIXED = 1, MA_PREC_FP64_FMA = 2 };
enum { MA_GATHER_ATOMICS = 0, MA_GATHER_CELL_FLUX = 1 };
/* State layouts: AOS is View<double*[5]> LayoutRight (U[c*5+k], the
 * reference's host layout); SOA is U[k*ncells+c]. */
enum { MA_LAYOUT_AOS = 0, MA_LAYOUT_SOA = 1 };
/* Initial conditions. */
enum { MA_IC_REFERENCE = 0, MA_IC_SOD = 1, MA_IC_CONSTANT = 2 };

/* Run options: the nine values of miniaero.inp (kokkos/Options.h:47-102)
 * followed by extension keys the reference hard-codes. */
typedef struct {
  int32_t problem_type;       /* 0 Sod, 1 viscous flat plate, 2 inviscid ramp */
  double lx, ly, lz, angle;
  int32_t nx, ny, nz;
  int32_t ntimesteps;
  double dt;
  int32_t output_results;
  int32_t output_frequency;
  int32_t second_order_space;
  int32_t viscous;
  /* extensions (defaults reproduce the reference) */
  int32_t limiter;            /* MA_LIMITER_*; reference: Venkatakrishnan */
  int32_t viscosity_model;    /* MA_VISC_*; reference: Sutherland, Pr 0.71 */
  double mu;                  /* constant viscosity */
  double prandtl;             /* Prandtl number for the constant model */
  int32_t precision;          /* MA_PREC_* */
  double cfl;                 /* > 0: dt = cfl * min_c V_c / sum_f(|u.n| + c|n|) at t = 0 */
  int32_t ic;                 /* MA_IC_* */
  double sod_left[2];         /* (rho, p) left of the split (MA_IC_SOD) */
  double sod_right[2];        /* (rho, p) right of the split */
  double sod_split;           /* split position in x; <= 0 means lx/2 */
  int32_t inflow_given;       /* 1: use inflow_state below */
  double inflow_state[5];     /* conserved inflow / constant state */
  int32_t bc_override[6];     /* per side (bottom, top, front, back, right, left), -1 = default map */
  int32_t keep_residual;      /* 1: keep the last stage residual on the device */
  int32_t gather;             /* MA_GATHER_*: the reference's default -DATOMICS_FLUX
                                 reduction order, or its -DCELL_FLUX build (per-slot
                                 storage summed in slot order; needs a mesh uploaded
                                 with MA_MESH_CELL_FLUX) */
} ma_options;

/* One face list; mirrors Faces<Device> (kokkos/Faces.h:42-71). Vector
 * fields are [nfaces*3] row-major, conn and flux_index [nfaces*2]. */
typedef struct {
  int32_t nfaces;
  int32_t type;               /* MA_BC_* for boundary sets, -1 for internal */
  const int32_t* conn;        /* (elem1, elem2); elem2 = -1 on the boundary */
  const int32_t* flux_index;  /* may be NULL */
  const double* coords;
  const double* normal;
  const double* tangent;
  const double* binormal;
  const int32_t* permutation; /* iteration order (Faces::permute_vector_) */
} ma_face_set;

#define MA_MAX_BC_SETS 16

/* A mesh as the reference's MeshData holds it (kokkos/MeshData.h:42-58). */
typedef struct {
  int32_t ncells;
  const double* cell_coords;  /* [ncells*3] */
  const double* cell_volumes; /* [ncells] */
  ma_face_set internal;
  int32_t nbc;
  ma_face_set bc[MA_MAX_BC_SETS]; /* boundary_faces order */
} ma_mesh_view;

typedef struct ma_host_mesh ma_host_mesh;
typedef struct ma_mesh ma_mesh;
typedef struct ma_solver ma_solver;

/* ---- library ------------------------------------------------------------ */
int32_t ma_abi_version(void);
const char* ma_last_error(void);
const char* ma_status_string(ma_status s);
/* Number of CUDA devices visible (0 without a GPU). */
int32_t ma_device_count(void);

/* ---- options ------------------------------------------------------------ */
/* Defaults of Options::Options() (kokkos/Options.h:59-69) plus extensions. */
void ma_options_default(ma_options* o);
/* Options::read_options_file (kokkos/Options.h:73-101): reads the nine
 * positional values, then optional "key value" extension lines. Unlike the
 * reference, a missing file or a malformed value is an error (MA_EIO /
 * MA_EINVAL), not a silent default. */
ma_status ma_options_read(const char* path, ma_options* o);

/* ---- run controls and checkpoints ---------------------------------------
 * No counterpart in the reference, whose only output is results.<rank>
 * (TimeSolverExplicitRK4.h:514-538). Run controls are extra lines of the same
 * input file, one per line ("checkpoint <path>", "checkpoint_frequency <n>",
 * "restart <path>"); ma_options_read skips them. */
#define MA_PATH_MAX 512
typedef struct {
  char checkpoint_path[MA_PATH_MAX];  /* "" = no checkpoints */
  int32_t checkpoint_frequency;       /* steps between checkpoints; 0 = only at the end */
  char restart_path[MA_PATH_MAX];     /* "" = start from the initial conditions */
} ma_run_options;
void ma_run_options_default(ma_run_options* r);
ma_status ma_run_options_read(const char* path, ma_run_options* r);

typedef struct {
  int64_t ncells;
  int64_t steps_done;   /* RK4 steps behind the state */
  double time;          /* simulated time of the state */
  double dt;            /* the run's time step (restarts keep it) */
  uint64_t mesh_hash;   /* ma_mesh_hash of the mesh the state belongs to */
} ma_checkpoint_info;
/* 64-bit hash of a mesh's cell count, cell centroids and volumes, and face
 * set sizes and types: a restart checks it against the checkpoint's. */
uint64_t ma_mesh_hash(const ma_mesh_view* view);
/* Writes the conserved state U (ncells x 5 in `layout`) with its header and
 * a payload checksum; the file appears under `path` only once complete. */
ma_status ma_checkpoint_write(const char* path, const ma_checkpoint_info* info, const double* U, int32_t layout);
/* Reads the header into *info and, when U is not NULL, the state (at most
 * max_cells cells) in `layout`. MA_EIO: unreadable, truncated or checksum
 * mismatch; MA_EINVAL: not a checkpoint, other version, too many cells. */
ma_status ma_checkpoint_read(const char* path, ma_checkpoint_info* info, double* U, int64_t max_cells,
                             int32_t layout);

/* ---- host mesh (replaces Parallel3DMesh + MeshProcessor, single rank) ---- */
/* Parallel3DMesh::Parallel3DMesh + fillMeshData (kokkos/Parallel3DMesh.C:36,
 * Parallel3DMesh.h:173-449): builds cells, faces, BC sets and the face
 * iteration permutations on the host. */
ma_status ma_host_mesh_build(const ma_options* o, ma_host_mesh** out);
/* As ma_host_mesh_build; with MA_HOST_MESH_DEVICE_GEOMETRY the per-face
 * geometry (kokkos/Face.C:37-98) and the cell volumes and centroids
 * (MeshProcessor.C:130-171) are computed on the current CUDA device,
 * bit-identical to the host path; face order, shuffle and BinSort stay on
 * the host. MA_ECUDA if the device cannot be used. */
enum { MA_HOST_MESH_DEVICE_GEOMETRY = 1 };
ma_status ma_host_mesh_build_ex(const ma_options* o, int32_t flags, ma_host_mesh** out);
ma_status ma_host_mesh_view(const ma_host_mesh* m, ma_mesh_view* view);
void ma_host_mesh_free(ma_host_mesh* m);
/* Initial state on the host (kokkos/Initial_Conditions.h:38-133), U in AOS. */
ma_status ma_host_initial_state(const ma_host_mesh* m, const ma_options* o, double* U);

/* ---- device mesh (replaces copy_faces / copy_cell_data, Faces.h:88,
 *      Cells.h:127) --------------------------------------------------------- */
/* Uploads any mesh given as ma_mesh_view: builds the device face order, the
 * per-face Roe frame and the per-cell ordered contribution lists that replay
 * the reference's serial accumulation order. At most MA_MAX_MESH_CELLS cells
 * (the device arrays use 32-bit indices; MA_EINVAL beyond) and fewer than
 * 2^30 faces. */
#define MA_MAX_MESH_CELLS 143165576
ma_status ma_mesh_upload(const ma_mesh_view* view, ma_mesh** out);
/* As ma_mesh_upload; flags MA_MESH_CELL_FLUX also builds the per-cell lists
 * in element-local slot order (from every face set's flux_index) that
 * solvers and batches with gather = MA_GATHER_CELL_FLUX use (72 more bytes
 * per cell). No reference counterpart as a call: it stands for the
 * reference's compile-time choice of -DCELL_FLUX. */
#define MA_MESH_CELL_FLUX 1
ma_status ma_mesh_upload_ex(const ma_mesh_view* view, int32_t flags, ma_mesh** out);
void ma_mesh_free(ma_mesh* m);
/* Device bytes held by the mesh. */
size_t ma_mesh_device_bytes(const ma_mesh* m);

/* ---- solver (replaces TimeSolverExplicitRK4, TimeSolverExplicitRK4.h:164) */
/* TimeSolverExplicitRK4(MeshData&, const Options&). dt comes from o->dt, or
 * from o->cfl when > 0 (evaluated on the state given to set_state / init). */
ma_status ma_solver_create(ma_mesh* mesh, const ma_options* o, ma_solver** out);
void ma_solver_free(ma_solver* s);
/* Initial conditions of Solve() (TimeSolverExplicitRK4.h:324-336). */
ma_status ma_solver_init_state(ma_solver* s, const ma_host_mesh* host_mesh);
ma_status ma_solver_set_state(ma_solver* s, const double* U, int32_t layout);
ma_status ma_solver_get_state(ma_solver* s, double* U, int32_t layout);
/* Residual of the last stage (Solve's res_vec); needs keep_residual. */
ma_status ma_solver_get_residual(ma_solver* s, double* res, int32_t layout);
/* nsteps RK4 steps (the body of Solve's time loop, :340-491), asynchronous
 * on the solver's stream. */
ma_status ma_solver_step(ma_solver* s, int32_t nsteps);
ma_status ma_solver_synchronize(ma_solver* s);
/* Kernel kinds reported by ma_solver_profile_steps. */
#define MA_PROFILE_KINDS 4
enum { MA_KERNEL_SWEEP = 0,          /* gradient + min/max + limiter, per cell */
       MA_KERNEL_INTERNAL_FLUX = 1,  /* Roe + viscous flux, per internal face */
       MA_KERNEL_BC_FLUX = 2,        /* boundary-face flux */
       MA_KERNEL_RESIDUAL = 3 };     /* ordered gather + RK4 update, per cell */
/* Advances nsteps steps like ma_solver_step but launching kernels one by one
 * with CUDA events around each on the solver's stream; returns the summed
 * milliseconds and launch counts per kernel kind (arrays of MA_PROFILE_KINDS). */
ma_status ma_solver_profile_steps(ma_solver* s, int32_t nsteps, double* kernel_ms, int32_t* kernel_launches);
/* The solver's cudaStream_t, for event timing by the caller. */
void* ma_solver_stream(ma_solver* s);
double ma_solver_dt(const ma_solver* s);
int64_t ma_solver_steps_done(const ma_solver* s);
/* Kernel launches issued per RK4 step (for launch accounting). */
int32_t ma_solver_launches_per_step(const ma_solver* s);
/* Sets dt explicitly (after create). */
ma_status ma_solver_set_dt(ma_solver* s, double dt);
/* Checks the state for non-finite values or non-positive density/energy;
 * returns MA_ENUMERIC and the first bad cell in *bad_cell if found. */
ma_status ma_solver_check_state(ma_solver* s, int64_t* bad_cell);
/* One full solve as the reference's Solve(): init + ntimesteps steps. */
ma_status ma_solver_solve(ma_solver* s, const ma_host_mesh* host_mesh);

/* Allocation-free CFL time step. No counterpart in the reference, which takes
 * dt from the input file. For callers that cannot allocate device memory at
 * that point (all memory handed to their own pool, or a loop that must not
 * block on the allocator): *dt_out = cfl * min_c V_c / sum_f(|u.n| + c|n|),
 * the value ma_solver_set_state computes, from the device state d_state
 * (conserved, [5][C] doubles, component-major) on the mesh, with kernels on
 * `stream` (a cudaStream_t, NULL = legacy default); returns after the stream
 * has reached the result. Scratch is a fixed 512 KiB array inside the
 * library; nothing is allocated. Meshes above 16,777,216 cells get MA_EINVAL.
 * The call runs on the mesh's device (the caller's current device is restored
 * afterwards); d_state must be on that device. It synchronises `stream` to
 * read dt back, so it must not be called on a stream that is being captured.
 * The first call on a device sets up the scratch address and keeps it for the
 * process (make that call before any global-mode capture on other streams; a
 * cudaDeviceReset of the device invalidates it). Calls that overlap on the
 * GPU share the scratch and race. */
ma_status ma_cfl_dt_noalloc(const ma_mesh* mesh, const double* d_state, double cfl, double* dt_out, void* stream);

/* ---- batched multi-mesh solver ------------------------------------------
 * No reference counterpart as an API: the reference advances one mesh per
 * process (Solve(), TimeSolverExplicitRK4.h:206) and scales out with MPI
 * ranks; here independent meshes of uneven size share one device and advance
 * together, one persistent launch per kernel kind and stage for the whole
 * batch, captured in a CUDA graph. Physics options (order, viscosity,
 * limiter, precision) are per batch; time step and inflow state per member.
 * A member's result is bit-identical to the same solve run alone. */
typedef struct ma_batch ma_batch;
/* capacity: maximum members; budget_bytes: device bytes members may hold. */
ma_status ma_batch_create(const ma_options* physics, int32_t capacity, size_t budget_bytes, ma_batch** out);
void ma_batch_free(ma_batch* b);
/* Device bytes a member on this mesh would hold (budget accounting). */
size_t ma_batch_member_bytes(const ma_batch* b, const ma_mesh* mesh);
/* Adds a member with initial state U0. dt > 0 fixes the time step; dt <= 0
 * takes it from physics->cfl on U0. inflow_state (5 conserved values) may be
 * NULL for physics->inflow_state. MA_EBUDGET when it does not fit. The mesh
 * must outlive the member. */
ma_status ma_batch_add(ma_batch* b, ma_mesh* mesh, const double* U0, int32_t layout, double dt,
                       const double* inflow_state, int32_t* member_id);
ma_status ma_batch_remove(ma_batch* b, int32_t member_id);
ma_status ma_batch_get_state(ma_batch* b, int32_t member_id, double* U, int32_t layout);
/* Advances every member nsteps RK4 steps (asynchronous). */
ma_status ma_batch_step(ma_batch* b, int32_t nsteps);
/* Single-launch mode: with block > 0 (64..256, a multiple of 32), every
 * ma_batch_step(b, n) runs all n RK4 steps of every member as ONE
 * cooperative kernel launch of `block` threads x as many blocks as fit on the
 * device at once (written to *grid_out when not NULL): the stage kernels
 * become phases of one persistent kernel, separated by a grid barrier whose
 * waits are bounded (ma_batch_synchronize then returns MA_ETIMEDOUT). Every
 * kind's chunks take `block` items. Same bits as the per-kind launches;
 * block = 0 returns to those (captured in a CUDA graph per step). */
ma_status ma_batch_set_single_launch(ma_batch* b, int32_t block, int32_t* grid_out);
ma_status ma_batch_synchronize(ma_batch* b);
void* ma_batch_stream(ma_batch* b);
int64_t ma_batch_cells(ma_batch* b);
int32_t ma_batch_size(const ma_batch* b);
size_t ma_batch_device_bytes(const ma_batch* b);
int64_t ma_batch_member_steps(const ma_batch* b, int32_t member_id);
double ma_batch_member_dt(const ma_batch* b, int32_t member_id);
/* Launch shapes per kernel kind (MA_KERNEL_*): threads per block (= items per
 * chunk) and persistent grid size. */
ma_status ma_batch_get_launch(const ma_batch* b, int32_t* block, int32_t* grid);
ma_status ma_batch_set_launch(ma_batch* b, const int32_t* block, const int32_t* grid);
/* Autotuner: times each kernel kind over the current members for block sizes
 * 64/128/256 x 1..16 CTAs per SM and keeps the fastest; member states are
 * restored afterwards. best_ms (4 values, may be NULL) receives the chosen
 * per-launch times. */
ma_status ma_batch_autotune(ma_batch* b, int32_t reps, double* best_ms);
/* Advances every member nsteps steps like ma_batch_step, but launching the
 * kernels one by one (no graph) with CUDA events around each on the batch's
 * stream; returns summed milliseconds and launch counts per kernel kind
 * (arrays of MA_PROFILE_KINDS). */
ma_status ma_batch_profile_steps(ma_batch* b, int32_t nsteps, double* kernel_ms, int32_t* kernel_launches);

/* ---- serving loop -------------------------------------------------------
 * No reference counterpart: the reference runs one solve per invocation
 * (Main.C:96-151). The server admits solve requests first-in first-out while
 * their device memory (member state + cached device mesh) fits the budget,
 * keeps their state resident, and advances all running requests together in
 * ticks of the batch solver (continuous batching: arrivals join at the next
 * tick, finished requests leave). Every request's result equals the same
 * solve run alone. */
typedef struct ma_server ma_server;
enum { MA_SERVER_THREAD = 1,   /* run the scheduling loop on a server thread */
       MA_SERVER_DRYRUN = 2 }; /* no device work: sizes and ticks only (host tests) */
enum { MA_REQ_QUEUED = 0, MA_REQ_RUNNING = 1, MA_REQ_DONE = 2, MA_REQ_CANCELLED = 3, MA_REQ_FAILED = 4 };
typedef struct {
  int32_t nx, ny, nz;          /* box mesh cells per axis */
  int32_t problem_type;        /* selects the BC map (Parallel3DMesh.h:382-396) */
  double lx, ly, lz, angle;
  double inflow_state[5];      /* conserved inflow state, also the initial state */
  int32_t nsteps;              /* RK4 steps to run */
  double dt;                   /* > 0: fixed; <= 0: from the server's physics.cfl */
  int32_t keep_result;         /* 1: keep the final state for ma_server_result */
} ma_request;
typedef struct {
  int32_t state;               /* MA_REQ_* */
  int32_t error;               /* ma_status of a failed request */
  int64_t steps_done;
  int64_t cells;
  int64_t t_submit_ns, t_admit_ns, t_finish_ns;  /* since server creation */
  double state_sq_norm[5];     /* sum over cells of U_k^2 of the final state */
} ma_request_info;
typedef struct {
  int64_t submitted, admitted, completed, failed, cancelled;
  int64_t ticks, cell_stages;
  int64_t bytes_in_use, peak_bytes;
  int32_t running, queued, peak_running, capacity, cached_meshes;
  double busy_seconds;         /* time with at least one request running */
} ma_server_stats;
/* physics: options shared by all requests (order, viscosity, limiter,
 * precision, cfl); budget_bytes: device bytes for states and meshes;
 * tick_steps: RK4 steps per scheduling tick; capacity: max running requests. */
ma_status ma_server_create(const ma_options* physics, size_t budget_bytes, int32_t tick_steps, int32_t capacity,
                           int32_t flags, ma_server** out);
void ma_server_free(ma_server* s);
/* Admission cap on the cells of running requests (0 = none; default). A
 * request larger than the cap still runs when nothing else does. */
ma_status ma_server_set_max_running_cells(ma_server* s, int64_t cells);
/* Launch shapes of the server's batch (as ma_batch_set_launch), e.g. the ones
 * ma_batch_autotune found for the workload; only while no request is queued
 * or running (MA_ESTATE otherwise). */
ma_status ma_server_set_launch(ma_server* s, const int32_t* block, const int32_t* grid);
/* Thread-safe; returns at once with the request id. */
ma_status ma_server_submit(ma_server* s, const ma_request* r, int64_t* id);
/* Builds and caches the device mesh a request of this shape would use. */
ma_status ma_server_preload_mesh(ma_server* s, const ma_request* r);
/* One scheduling iteration (admit, tick, retire) when the server has no
 * thread of its own; *progressed = 0 when nothing ran. */
ma_status ma_server_poll(ma_server* s, int32_t* progressed);
ma_status ma_server_cancel(ma_server* s, int64_t id);
ma_status ma_server_query(ma_server* s, int64_t id, ma_request_info* info);
/* Final state (AOS) of a finished request that set keep_result. */
ma_status ma_server_result(ma_server* s, int64_t id, double* U);
/* Waits until the request leaves the queue/running states or timeout_s
 * passes (MA_ETIMEDOUT). Without a server thread it drives the loop itself. */
ma_status ma_server_wait(ma_server* s, int64_t id, double timeout_s);
ma_status ma_server_get_stats(ma_server* s, ma_server_stats* out);

/* ---- diagnostics (host only) -------------------------------------------- */
/* First n outputs of the glibc rand() sequence for seed (the generator behind
 * std::random_shuffle in Parallel3DMesh.h:362). */
ma_status ma_debug_glibc_rand(uint32_t seed, int32_t n, int32_t* out);
/* Serial Kokkos BinSort permutation of keys (Faces.h:128-144). */
ma_status ma_debug_binsort(const int32_t* keys, int32_t n, int32_t* perm);

/* Checks the device's reciprocal-based correctly rounded division against
 * IEEE division on n generated pairs (mode 0 random, 1 divisors with an
 * all-ones significand, 2 quotients near rounding midpoints); mode 3 checks
 * the integer float->double widening of the mixed form instead, mode 4 its
 * integer double->float rounding; mode 5 divides tiny, subnormal and zero
 * numerators; mode 6 checks the FP64 identities the plain form evaluates with
 * integer instructions (0.5*x, 2*x, 0+x, |x|, and x < y for a non-negative x)
 * against the FP64 instructions, over every exponent class. Returns the
 * mismatch count and, if any, one failing pair in example[0..1]. */
ma_status ma_debug_check_division(int32_t mode, uint64_t n, uint64_t seed, uint64_t* mismatches, double* example);

/* Measured FP64 issue rate of this device (thread instructions per second):
 * op 0 additions, 1 multiplications, 2 fused multiply-adds, each as 4
 * independent chains per thread on 8 blocks of 256 threads per SM; the best
 * of 3 timed launches after one warm-up. The ceiling the FP64 form's kernels
 * are measured against. */
ma_status ma_debug_fp64_rate(int32_t op, double* inst_per_s);

/* Failure path of the grid barrier that separates the phases of the batch's
 * single-launch step (ma_batch_set_single_launch): a cooperative launch of 2
 * blocks in which block 1 returns at once, so block 0's wait at the barrier
 * runs out after timeout_s (at most 10 s) instead of completing. Returns
 * whether block 0 passed the barrier (*passed, 0 expected), the error word
 * it left (*error_word, 1 expected) and the host-measured duration. The
 * device context stays usable. */
ma_status ma_debug_barrier_timeout(double timeout_s, int32_t* passed, int32_t* error_word, double* waited_s);

/* ---- operator-level entry points (unit parity; host arrays in and out) --- */
/* roe_flux::compute_flux (Roe_Flux.h:50) on n independent faces:
 * pl, pr [n*5] primitives; normal, tangent, binormal [n*3]; flux [n*5]. */
ma_status ma_op_roe_flux(int32_t n, const double* pl, const double* pr, const double* normal,
                         const double* tangent, const double* binormal, double* flux);
/* newtonian_viscous_flux::compute_flux (Viscous_Flux.h:66): grad [n*15]
 * (component-major 5x3), prim [n*5], area [n*3], vflux [n*5]. */
ma_status ma_op_viscous_flux(int32_t n, const double* grad, const double* prim, const double* area,
                             int32_t viscosity_model, double mu, double prandtl, double* vflux);
/* VenkatLimiter::limit (VenkatLimiter.h:45) or VanAlbadaLimiter::limit
 * (VanAlbadaLimiter.h:45), element-wise over n values (d2 ignored by Van Albada). */
ma_status ma_op_limiter(int32_t n, int32_t kind, const double* dumax, const double* dumin,
                        const double* du, const double* d2, double* phi);
/* ComputePrimitives (GasModel.h:69), U and V [n*5]. */
ma_status ma_op_primitives(int32_t n, const double* U, double* V);

/* One RK stage's drivers taken one at a time on an uploaded mesh and a
 * conserved state U (ncells x 5 in `layout`), in the reference's serial
 * (ATOMICS_FLUX) order; outputs are cell-major like the reference's host
 * views. The solver runs the same kernels fused into its four per stage. */
/* GreenGauss::compute_gradients (GreenGauss.h:300-321): gradients of the
 * primitives, grad [ncells*15] as (cell, component, direction). */
ma_status ma_op_green_gauss(ma_mesh* mesh, const double* U, int32_t layout, double* grad);
/* StencilLimiter::compute_min_max + compute_limiter (StencilLimiter.h:532-616)
 * with the Green-Gauss gradient of the same U and limiter MA_LIMITER_*:
 * phi [ncells*5]. */
ma_status ma_op_stencil_limiter(ma_mesh* mesh, int32_t limiter, const double* U, int32_t layout, double* phi);
/* The boundary functors compute_{extrapolate,tangent,NoSlip,inflow}BC_flux as
 * Solve applies them (TimeSolverExplicitRK4.h:428-475): each cell's boundary
 * contributions to cell_flux, summed from zero, [ncells*5]. o supplies the
 * viscosity model (NoSlip is always viscous) and the inflow state. */
ma_status ma_op_bc_flux(ma_mesh* mesh, const ma_options* o, const double* U, int32_t layout, double* cell_flux);
/* apply_cell_flux (Flux.h:188-229): res = 0 + (dt / V) * cell_flux, [ncells*5]. */
ma_status ma_op_apply_cell_flux(int32_t ncells, double dt, const double* volumes, const double* cell_flux,
                                double* res);
/* update (TimeSolverExplicitRK4.h:106-128): dst = src + alpha * res over n values. */
ma_status ma_op_rk_update(int64_t n, double alpha, const double* res, const double* src, double* dst);

#ifdef __cplusplus
}
#endif
#endif
