/*
 * luxum.h -- C ABI of the GB300 FDTD engine (drop-in for Luxum's time-stepping path).
 *
 * Plain C: no C++ types, no torch types, no exceptions cross this boundary.  Every call
 * returns an lx_status (0 = ok); the text of the last failure is available through
 * lx_last_error(sim) (per handle) or lx_last_error(NULL) (per thread, for calls that
 * failed before a handle existed).
 *
 * What each entry point replaces in the reference (paths are within the Luxum project):
 *   lx_params / lx_params_init / lx_params_from_yaml
 *       -> class reader: public members reader.h:50-174, readYAML() reader.cc:68-130,
 *          checkData() reader.cc:141-162 (the reader constructor reader.cc:55-58 runs both)
 *   lx_sim_create
 *       -> grid::grid grid.cc:58-95 (single rank: local = global), maxwell::maxwell
 *          maxwell.cc:60-148 (constants, PML and plane-wave set-up, plane_wave_initialise
 *          maxwell.cc:825-929), the vfield/field allocations of the four drivers
 *          (two_dim.cc:63-68, two_dim_pml.cc:86-106, three_dim.cc:66-72,
 *          three_dim_pml.cc:92-107) and the CPML profiles k_fn/b_fn/c_fn maxwell.cc:997-1280
 *   lx_sim_set_cb / lx_sim_set_material
 *       -> the Cb coefficient set-up of the drivers: Cb = dt/eps0 (two_dim.cc:81,
 *          two_dim_pml.cc:116, three_dim.cc:54) and the material-file formula
 *          Cb = dt/(eps0*(1+F*1e6)) (three_dim_pml.cc:109-128, fileio::readHDF5 fileio.cc:224-247)
 *   lx_sim_step
 *       -> one iteration of the time loop of maxwell::solve() maxwell.cc:157-174:
 *          solve_planar two_dim.cc:85-144, solve_planar_pml two_dim_pml.cc:126-188,
 *          solve3d three_dim.cc:82-196, solve3d_pml three_dim_pml.cc:158-283
 *          (curl vfield.cc:102-386, TF/SF plane_wave_execute maxwell.cc:194-812,
 *          point source maxwell.cc:944-979 + drivers, max|E|^2 monitor)
 *   lx_sim_read_field / lx_sim_write_field / lx_sim_field_shape
 *       -> field::F of each component (field.h:54, staggered extents field.cc:58-77)
 *   lx_sim_max_e2
 *       -> local_max / MPI_Reduce(MAX) of the drivers (two_dim_pml.cc:136,181,
 *          three_dim_pml.cc:168,266-276)
 *   lx_sim_set_snapshots / lx_sim_set_hdf5_output / lx_sim_sync
 *       -> fileio(name,false,grid,field*) + writeHDF5(t) fileio.cc:60-212 and the drivers'
 *          "t % n == 0" write cadence (two_dim_pml.cc:184, three_dim_pml.cc:279)
 *
 * Ownership: the library owns all device memory of a handle; callers own every host
 * buffer they pass.  Distinct handles may be used from distinct host threads; one handle
 * must not be used from two threads at once.
 */
#ifndef LUXUM_H
#define LUXUM_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__) && defined(LX_BUILDING_LIBRARY)
#define LX_API __attribute__((visibility("default")))
#else
#define LX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lx_status {
  LX_OK = 0,
  LX_ERR_INVALID = 1,     /* bad argument or parameter combination */
  LX_ERR_UNSUPPORTED = 2, /* a combination the reference cannot run either (see message) */
  LX_ERR_CUDA = 3,        /* a CUDA call failed */
  LX_ERR_OOM = 4,         /* device or pinned host allocation failed */
  LX_ERR_BLOWUP = 5,      /* max|E|^2 became non-finite */
  LX_ERR_IO = 6,          /* file open/parse/write failure */
  LX_ERR_STATE = 7        /* call not valid in the handle's current state */
} lx_status;

/* Storage/compute precision of the fields (engine option; the reference is FP64 only). */
enum { LX_PREC_FP64 = 0, LX_PREC_FP32 = 1, LX_PREC_FP16S = 2 };
/* CPML coefficient b: reference form exp(-(sigma/kappa - a)/eps0*dt) (maxwell.cc:1215)
 * or the textbook form exp(-(sigma/kappa + a)/eps0*dt). */
enum { LX_CPML_REFERENCE = 0, LX_CPML_STANDARD = 1 };
/* Point-source waveform: the reference's hard CW source amp*sin(omega*t*dt) with amp and
 * omega truncated to int (maxwell.h:203,206; three_dim_pml.cc:161-165), or an additive
 * Gaussian-modulated sine pulse amp*exp(-((t-t0)/tw)^2)*sin(omega*t*dt). */
enum { LX_SRC_CW_HARD = 0, LX_SRC_PULSE_SOFT = 1 };
/* Field components, in the reference's vfield order (vfield.cc:58-87). */
enum { LX_EX = 0, LX_EY = 1, LX_EZ = 2, LX_HX = 3, LX_HY = 4, LX_HZ = 5, LX_ETOTAL = 6 };

/* Mirrors the public members of class reader (reader.h:50-174) in parameters.yaml order,
 * followed by engine options that have no YAML key in the reference. */
typedef struct lx_params {
  /* document 1: "isPlanar" */
  int isPlanar;
  /* document 2: "X/Y/Z Length", "X/Y/Z Resolution", "Courant factor", "Number of timesteps" */
  int Nx, Ny, Nz;
  double dx, dy, dz;
  double S;
  int num_timesteps;
  /* document 3: "X/Y Number of Procs", "Number of Threads per node".  Validated like
   * reader::checkData; one GPU holds the whole grid, so they do not split it. */
  int npX, npY, n_threads;
  /* document 4: sources */
  int usePS;
  int Nx_source, Ny_source, Nz_source;
  double amp_source, omega_source;
  int usePW;
  double kx_pw, ky_pw, kz_pw;
  double Ex_pw, Ey_pw, Ez_pw;
  double off_pw;
  int x1_pw, y1_pw, z1_pw, x2_pw, y2_pw, z2_pw;
  /* document 5: boundary conditions */
  int usePML;
  double d_pml;   /* "Thickness of PML" (metres) */
  double sigma;   /* "sigma_max/sigma_optimal" (reader::sigma) */
  double sigma_m; /* "m value of sigma" */
  double kappa;   /* "kappa max" */
  double a_max;   /* "max value of a" */
  double a_m;     /* "m value for a" */
  /* engine options (defaults from lx_params_init reproduce the reference) */
  int precision;      /* LX_PREC_* (default FP64) */
  double pw_sigma;    /* plane-wave pulse width in m^2 (default pow(10,-4)/0.5, maxwell.cc:71) */
  int cpml_mode;      /* LX_CPML_* (default LX_CPML_REFERENCE) */
  int source_kind;    /* LX_SRC_* (default LX_SRC_CW_HARD) */
  double src_t0;      /* LX_SRC_PULSE_SOFT: pulse centre in steps */
  double src_tw;      /* LX_SRC_PULSE_SOFT: pulse 1/e half-width in steps */
  int monitor_every;  /* compute max|E|^2 every n steps; 0 = only at the end of each lx_sim_step call */
} lx_params;

typedef struct lx_sim lx_sim;

/* Fills *p with the reference's defaults for everything not read from YAML. */
LX_API void lx_params_init(lx_params* p);

/* Parses a Luxum parameters.yaml (five flow-mapping documents, reader.cc:68-130) and runs
 * the checks of reader::checkData (reader.cc:141-162).  Optional sixth document: engine
 * options ("precision", "pulse width", "cpml mode", ...). */
LX_API lx_status lx_params_from_yaml(const char* path, lx_params* p);

/* Validates *p (reader::checkData plus the index ranges the reference reads out of bounds),
 * allocates all device state (fields zeroed as field.cc:78-85 does) and computes the
 * constants and CPML profiles exactly as maxwell.cc:60-148 / 997-1280. */
LX_API lx_status lx_sim_create(const lx_params* p, lx_sim** out);
LX_API void lx_sim_destroy(lx_sim* sim);
/* Device memory lx_sim_create would hold for *p (fields, coefficients, CPML psi slabs and
 * profiles, TF/SF tables), computed on the host without a GPU; snapshot staging, probes,
 * DFT planes and transfer buffers come on top when used.  Serving loops admit requests
 * against an HBM budget with it. */
LX_API lx_status lx_params_device_bytes(const lx_params* p, size_t* bytes);
/* Compulsory device-memory traffic of one time step for *p, computed on the host: every
 * field component read and written once, every Cb array read once and every stored CPML psi
 * entry read and written once, over the Nx*Ny*Nz cells (padding excluded), at the storage
 * sizes of p->precision.  The figure a roofline divides by the step time.  Measurement aid
 * with no counterpart in the reference (whose drivers move about four times as much). */
LX_API lx_status lx_params_step_bytes(const lx_params* p, double* bytes);
/* Handles and batches take device memory from the current device's stream-ordered pool and
 * give it back there when destroyed, for reuse without a device-wide synchronisation.  This
 * waits for the device and returns the pool's unused memory to the driver. */
LX_API lx_status lx_trim_device_memory(void);
/* Zeroes E, H, psi and |E|^2 and rewinds to step 0 (the state after lx_sim_create); keeps
 * Cb, probe positions and snapshot outputs, so one handle can run many simulations. */
LX_API lx_status lx_sim_reset(lx_sim* sim);

/* Sets the Cb update coefficient of E component comp (LX_EX..LX_EZ; planar: LX_EY only)
 * from n = product of the component's staggered extents host doubles, C order. */
LX_API lx_status lx_sim_set_cb(lx_sim* sim, int comp, const double* cb, size_t n);
/* Cb = dt / (eps0 * (1 + F * scale)), the reference's material-file formula
 * (three_dim_pml.cc:122-128 with scale = 1e6; two_dim_pml.cc:112-113 with scale = 11). */
LX_API lx_status lx_sim_set_material(lx_sim* sim, int comp, const double* F, size_t n, double scale);
/* Cb = dt / (eps0 * eps_r) over an index box [lo, hi) of every E component. */
LX_API lx_status lx_sim_set_eps_box(lx_sim* sim, const int lo[3], const int hi[3], double eps_r);

/* Advances nsteps full Yee steps (H half-step then E half-step).  Blocks until the steps
 * are enqueued and, when a monitor step falls inside, until max|E|^2 is known. */
LX_API lx_status lx_sim_step(lx_sim* sim, int nsteps);
/* Waits for all queued device work and snapshot writes of the handle. */
LX_API lx_status lx_sim_sync(lx_sim* sim);

/* Staggered extents of a component (field.cc:67-77); absent planar components give 0s. */
LX_API lx_status lx_sim_field_shape(const lx_sim* sim, int comp, int shape[3]);
/* The same for the handle *p would give, on the host without a GPU (validates *p). */
LX_API lx_status lx_params_field_shape(const lx_params* p, int comp, int shape[3]);
LX_API lx_status lx_sim_read_field(lx_sim* sim, int comp, double* host, size_t n);
LX_API lx_status lx_sim_write_field(lx_sim* sim, int comp, const double* host, size_t n);
/* Same result as lx_sim_read_field, but the call allocates nothing: no cudaMalloc, cudaFree
 * or allocating library routine.  No counterpart in the reference.  It is meant for callers
 * that must not let a library allocate device memory at that point: processes whose GPU
 * memory is owned by another allocator (a framework caching allocator that has reserved
 * most of the device, where a new cudaMalloc fails or fragments its pool) and loops with
 * latency budgets (cudaMalloc/cudaFree can synchronise the device).  The component is
 * compacted through a fixed staging array of 1048576 doubles (8 MiB) that is part of the
 * library's static device memory; every GPU that loads the library holds it until the
 * process exits.  Components with more values than that are rejected with LX_ERR_INVALID
 * (use lx_sim_read_field).  The first call on a device looks up the array's device address
 * and caches it, so make that first call before any stream capture begins.  All calls on a
 * device share the array: calls whose GPU work overlaps (different streams or host threads
 * at once) race, so order them. */
LX_API lx_status lx_sim_read_field_noalloc(lx_sim* sim, int comp, double* host, size_t n);
/* Number of completed steps. */
LX_API int lx_sim_timestep(const lx_sim* sim);
/* max over the grid of Ey^2 (planar) or Ex^2+Ey^2+Ez^2 (3D) after the last monitor step. */
LX_API lx_status lx_sim_max_e2(lx_sim* sim, double* out);
/* The max|E|^2 of every monitored step (each step when monitor_every = 1; the last step of
 * each lx_sim_step call otherwise), kept on the device without a host round trip per step:
 * the series the reference drivers print, "t: <t>, max: <max>" (two_dim_pml.cc:135-141,
 * three_dim_pml.cc:168-175).  Up to `capacity` entries are kept between reads; later steps
 * still update lx_sim_max_e2 but are not recorded.  lx_sim_read_max_series returns the
 * steps and values recorded since the last read (*rows of them) and empties the series. */
LX_API lx_status lx_sim_set_max_series(lx_sim* sim, int capacity);
LX_API lx_status lx_sim_read_max_series(lx_sim* sim, int* steps, double* max_e2, int capacity, int* rows);

/* Point probes: every step records all six components at each (i,j,k) (0 where a
 * component's extent does not contain the index).  Replaces earlier probes. */
LX_API lx_status lx_sim_set_probes(lx_sim* sim, const int* ijk, int nprobes, int capacity_steps);
/* Copies [nsteps recorded][nprobes][6] doubles; *nsteps_out receives the row count. */
LX_API lx_status lx_sim_read_probes(lx_sim* sim, double* host, size_t n, int* nsteps_out);

/* Frequency-domain plane monitor (engine feature; the reference has none).  Keeps FP64
 * running DFTs, at nfreq angular frequencies omega[f] (rad/s), of the four field components
 * tangential to the plane normal to `axis` (0 x, 1 y, 2 z) through cell index `index`:
 * (E_t1, E_t2, H_t1, H_t2) with (t1, t2) = (y, z), (z, x) or (x, y).  After the E update of
 * every step t with t % every == 0 it adds every * E(t+1) e^{-i omega (t+1) dt} and
 * every * H(t+1/2) e^{-i omega (t+1/2) dt}; all four are sampled at the plane's cell (i,j,k)
 * (0 outside a component's extent).  Planar grids: the plane is a line, axis 0 or 2. */
LX_API lx_status lx_sim_add_dft_plane(lx_sim* sim, int axis, int index, int nfreq, const double* omega, int every,
                                      int* id);
/* Checkpoint / resume.  lx_sim_save writes the handle's whole state to one HDF5 file:
 * datasets "Ex".."Hz" in the layout of the snapshot files (staggered extents, C order,
 * physical values), then the per-cell Cb, the CPML psi slabs, the DFT accumulators and the
 * step counter.  lx_sim_load restores it into a handle created with the same parameters
 * (the step count, thread and process counts and monitor cadence may differ) and the same
 * DFT planes; the run then continues bit for bit as the saved one would have.  The probe
 * series restarts empty.  No reference counterpart (the reference cannot resume). */
LX_API lx_status lx_sim_save(lx_sim* sim, const char* path);
LX_API lx_status lx_sim_load(lx_sim* sim, const char* path);
/* Raw accumulators [nfreq][4][na][nb][2] (re, im), (na, nb) = in-plane extents in axis order. */
LX_API lx_status lx_sim_read_dft(lx_sim* sim, int id, double* host, size_t n);
/* Net power flux through the plane per frequency: sum over cells of
 * Re(E_t1 conj(H_t2) - E_t2 conj(H_t1)) times the cell face area (planar: the cell edge). */
LX_API lx_status lx_sim_dft_flux(lx_sim* sim, int id, double* flux, int nfreq);

/* Snapshot callback: called from the handle's writer thread, in step order, with a host
 * buffer valid only during the call. */
typedef void (*lx_snapshot_fn)(void* user, int timestep, int comp, const double* data,
                               const int shape[3]);
/* Every `every` steps (after the E update, when timestep % every == 0, as the drivers'
 * writeHDF5 cadence), copies the components in comp_mask (bit c = component c, bit 6 =
 * |E|^2 in the Ez-shaped array of three_dim_pml.cc:266-273) to pinned host memory on a
 * side stream and hands them to fn.  every = 0 disables. */
LX_API lx_status lx_sim_set_snapshots(lx_sim* sim, int every, unsigned comp_mask, lx_snapshot_fn fn,
                               void* user);
/* Adds an HDF5 file receiving component comp (LX_EX..LX_ETOTAL) at every step t with
 * t >= first and t % every == 0, in the layout of fileio.cc:60-212 (dataset "t=<step>",
 * global staggered dims, native double, contiguous).  The drivers' cadences: every 10
 * (two_dim_pml.cc:184), every 20 from 100 (two_dim.cc:140), |E|^2 every 10
 * (three_dim.cc:192) or every 3 (three_dim_pml.cc:279).  The file is complete after
 * lx_sim_destroy. */
LX_API lx_status lx_sim_set_hdf5_output(lx_sim* sim, int every, int first, int comp, const char* path);

/* HDF5 files in the reference's layout (host only, no GPU).  lx_hdf5_write creates `path`
 * with one 3-D native-double contiguous dataset per name (e.g. the material files that
 * three_dim_pml.cc:109-118 reads, dataset "data").  lx_hdf5_read reads a little-endian
 * float64/float32 dataset of rank <= 3 into `out` (n doubles, C order; out = NULL only
 * queries the shape); shape is right-aligned, so rank 2 gives {1, n0, n1}.  Files with
 * superblock 0/1, old-style groups and contiguous storage are supported (what fileio.cc
 * writes and what h5py writes by default); chunked or compressed datasets are not. */
LX_API lx_status lx_hdf5_write(const char* path, int ndatasets, const char* const* names, const double* const* data,
                               const int shape[3]);
LX_API lx_status lx_hdf5_read(const char* path, const char* dataset, double* out, size_t n, int shape[3]);

/* ---- batches: many independent simulations stepped together (engine feature) ----
 * Member handles keep their own device state; each step runs one prologue launch, one H and
 * one E launch per group of members sharing (planar, uniform spacing) over a tile table of
 * all of them, one launch for every member's DFT planes and a step-counter tick.  3-D
 * members of 2^18 cells or more instead take one H and one E launch each, spread over four
 * streams so that they overlap.  Members are updated in place (planar FP32/FP16 handles
 * move their state into their first buffer on joining).  From the second chunk
 * after a change of members on, chunks of steps are captured once as a CUDA graph and replayed
 * (the first is launched directly, so that a batch whose members change every chunk never
 * waits for a capture).  All members share one precision;
 * members may not have snapshot outputs or probes (use lx_sim_step for those).  max|E|^2
 * is monitored every step.  A handle belongs to at most one batch; lx_sim_step on a member
 * is allowed between batch steps (the batch re-reads its step counter). */
typedef struct lx_batch lx_batch;
LX_API lx_status lx_batch_create(lx_batch** out);
LX_API void lx_batch_destroy(lx_batch* b); /* does not destroy the members */
LX_API lx_status lx_batch_add(lx_batch* b, lx_sim* sim);
LX_API lx_status lx_batch_remove(lx_batch* b, lx_sim* sim);
LX_API int lx_batch_size(const lx_batch* b);
/* Steps between CUDA-graph captures (default 100; 0 launches without graphs). */
LX_API lx_status lx_batch_set_chunk(lx_batch* b, int steps);
/* Advances every member by nsteps; returns LX_ERR_BLOWUP if any member's max|E|^2 is not
 * finite afterwards (lx_last_error(NULL) names the first such member). */
LX_API lx_status lx_batch_step(lx_batch* b, int nsteps);
/* lx_batch_step in two halves: enqueue the steps and return at once, so the host can
 * prepare the next members while the GPU works; lx_batch_wait completes them (monitor
 * read-back, blow-up check).  Members must not be touched in between. */
LX_API lx_status lx_batch_step_async(lx_batch* b, int nsteps);
LX_API lx_status lx_batch_wait(lx_batch* b);
/* Tile shape of the batched update kernels: cells each thread walks along x, for planar
 * members (rows 8 apart) and for 3-D members below 2^18 cells (planes); each 1, 2, 4 or 8
 * (defaults 8, 8).  Results do not depend on it, only speed. */
LX_API lx_status lx_batch_set_march(lx_batch* b, int planar_rows, int planes_3d);
LX_API lx_status lx_batch_get_march(const lx_batch* b, int* planar_rows, int* planes_3d);
/* Tile-shape table.  Members are classed by (dimension, size, precision, CPML slab depth);
 * a class with an entry takes that entry's march, the others the per-dimension march above.
 * Members of different classes whose marches differ take separate launches. */
typedef struct lx_tune_entry {
  int planar;      /* 1 planar, 0 3-D */
  int size_class;  /* floor(log4(Nx*Ny*Nz)), at most 15 */
  int precision;   /* LX_PREC_* */
  int slab_class;  /* CPML slab depth along x: 0 none, 1 up to 8 cells, 2 up to 16, 3 deeper */
  int march;       /* 1, 2, 4 or 8 */
} lx_tune_entry;
/* Fills every field of *key but march with the handle's class. */
LX_API lx_status lx_sim_tune_class(const lx_sim* sim, lx_tune_entry* key);
/* Replaces the batch's table (n entries; n = 0 clears it).  Duplicate classes: the last wins. */
LX_API lx_status lx_batch_set_tune_table(lx_batch* b, const lx_tune_entry* entries, int n);
/* Copies up to cap entries to entries (may be NULL when cap is 0); *n = the table's length. */
LX_API lx_status lx_batch_get_tune_table(const lx_batch* b, lx_tune_entry* entries, int cap, int* n);
/* Tunes the class of every batched member (3-D members of 2^18 cells or more and planar
 * single-sweep members are launched one by one and have no tile shape).  Zero-field twins of
 * a sample of the members (up to 1.5e8 cells, at least one per class; created and freed here)
 * are stepped together, `steps` steps per timing: first with one march for every class, then
 * with each class in turn (largest first) moved to each other march, a move kept when the
 * whole sample runs 2 % faster, so that a class's pick pays for the launch it splits off.
 * Every class's pick is recorded in the table.  The members themselves are not stepped.  The
 * per-dimension march becomes the pick of the dimension's largest class and is reported. */
LX_API lx_status lx_batch_autotune(lx_batch* b, int steps, int* planar_rows, int* planes_3d);
/* Tunes the class of one handle (not necessarily a member yet) on zero-field twins of it,
 * replicated up to 2^24 cells or 64 twins, and records the pick; a march other than the
 * dimension's (lx_batch_set_march) must run 5 % faster.  *march = 0 when the class has no tile
 * shape.  The handle is not stepped.  Waits for the batch's enqueued steps. */
LX_API lx_status lx_batch_tune_member(lx_batch* b, const lx_sim* sim, int steps, int* march);

/* ---- Serving: continuous batching of submitted simulations --------------------------
 * No reference counterpart: the reference runs one simulation per process.  A server owns
 * one batch and a worker thread.  Requests queue in submission order; the worker admits
 * the head of the queue when its device memory fits the budget (or nothing is running),
 * creates its handle, and steps every running request together in chunks (lx_batch), so
 * requests join and leave between chunks without stopping the others.  A chunk never
 * overshoots a request's step count.  Handles for the next requests are created while a
 * chunk runs on the GPU.  All calls are thread-safe. */
typedef struct lx_server lx_server;
typedef struct lx_server_config {
  int precision;          /* LX_PREC_* shared by every request (default FP32) */
  int chunk;              /* steps per batch launch (default 100; captured as a CUDA graph when the
                             members did not change since the last chunk) */
  double budget_bytes;    /* device memory for running requests (default 0: 90% of free) */
  int max_running;        /* 0: no limit besides the budget */
  int tune_steps;         /* > 0: tune each new class of batched request on twins of it before
                             it joins (lx_batch_tune_member, `tune_steps` steps per march);
                             0 (default): no tuning while serving */
  const lx_tune_entry* tune_table;  /* tile shapes per request class to start from (copied at
                                       creation; e.g. from lx_batch_autotune on a sample of the
                                       expected requests), or NULL */
  int tune_entries;
} lx_server_config;
LX_API void lx_server_config_init(lx_server_config* cfg);

typedef struct lx_request {
  lx_params params;       /* params.precision must equal the server's */
  int steps;              /* time steps to run */
  /* material arrays F of E components LX_EX..LX_EZ (NULL: vacuum), each the component's
   * staggered extent in C order; Cb = dt/(eps0*(1+F*material_scale)) (lx_sim_set_material),
   * applied before the boxes */
  const double* material[3];
  double material_scale;
  int n_boxes;            /* dielectric boxes, applied in order (lx_sim_set_eps_box) */
  const int* boxes;       /* n_boxes x {lo[3], hi[3]} */
  const double* box_eps;  /* n_boxes relative permittivities */
  int dft_axis, dft_index, dft_every; /* one DFT plane (lx_sim_add_dft_plane) when nfreq > 0 */
  int nfreq;
  const double* omega;    /* nfreq angular frequencies */
} lx_request;
LX_API void lx_request_init(lx_request* r);

enum { LX_REQ_QUEUED = 0, LX_REQ_RUNNING = 1, LX_REQ_DONE = 2, LX_REQ_FAILED = 3, LX_REQ_CANCELLED = 4 };

typedef struct lx_server_stats {
  long long submitted, queued, running, done, failed, cancelled;
  double bytes_running;       /* device-memory estimate of the running requests */
  double peak_bytes_running;
  int peak_running;
  double cell_updates;        /* over all chunks stepped */
  double busy_seconds;        /* worker time with requests running */
  long long chunks;
  double tune_seconds;        /* worker time spent tuning classes (outside busy_seconds) */
  int tuned_classes;
  /* where the worker's time goes (seconds): enqueueing chunks (batch rebuilds and graph
   * captures included), creating request handles (inside chunks and between them), waiting
   * for chunks to finish after that, adding prepared handles to the batch, retiring requests */
  double enqueue_seconds, prepare_seconds, wait_seconds, join_seconds, retire_seconds;
} lx_server_stats;

LX_API lx_status lx_server_create(const lx_server_config* cfg, lx_server** out);
/* Stops the worker after the chunk in flight; running and queued requests are cancelled.
 * No other call on the same server may run concurrently with it. */
LX_API void lx_server_destroy(lx_server* srv);
/* Validates and copies the request (arrays included) and queues it; *id identifies it. */
LX_API lx_status lx_server_submit(lx_server* srv, const lx_request* req, long long* id);
LX_API lx_status lx_server_poll(lx_server* srv, long long id, int* state);
/* Waits until the request is DONE, FAILED or CANCELLED, or timeout_s passes (< 0: no
 * limit); *state is its state on return. */
LX_API lx_status lx_server_wait(lx_server* srv, long long id, double timeout_s, int* state);
/* Queued requests leave the queue; running ones leave the batch at the next chunk end. */
LX_API lx_status lx_server_cancel(lx_server* srv, long long id);
/* Results of a DONE request: the DFT plane's flux (lx_sim_dft_flux) and max|E|^2.  They
 * run without blocking the worker; take and release refuse a request while one runs. */
LX_API lx_status lx_server_flux(lx_server* srv, long long id, double* flux, int nfreq);
LX_API lx_status lx_server_max_e2(lx_server* srv, long long id, double* out);
/* Seconds since the server was created at which the request was submitted, started
 * running and finished (-1 where that has not happened). */
LX_API lx_status lx_server_times(lx_server* srv, long long id, double t[3]);
/* Hands the DONE request's handle to the caller (who then owns and destroys it) and
 * forgets the request. */
LX_API lx_status lx_server_take(lx_server* srv, long long id, lx_sim** sim);
/* Forgets a finished, failed or cancelled request and frees its handle. */
LX_API lx_status lx_server_release(lx_server* srv, long long id);
/* Why a request FAILED ("" otherwise); valid until the request is released. */
LX_API const char* lx_server_error(lx_server* srv, long long id);
LX_API lx_status lx_server_stats_get(lx_server* srv, lx_server_stats* st);
/* The server batch's tile-shape table (lx_batch_get_tune_table). */
LX_API lx_status lx_server_tune_table(lx_server* srv, lx_tune_entry* entries, int cap, int* n);

/* A batch is driven by one host thread at a time (the server's worker drives its own). */

/* Launch all device work of the handle on this CUDA stream (cudaStream_t) instead of its
 * own.  NULL restores the handle's own stream. */
LX_API lx_status lx_sim_set_stream(lx_sim* sim, void* cuda_stream);

/* Instrumented pass: runs nsteps steps with a CUDA event around every launch on the
 * handle's stream and returns the mean device time per launch in milliseconds of
 * out_ms[0] step prologue, [1] H-update kernel, [2] E-update kernel, [3] probe kernel
 * (0 when that kernel did not run).  Planar handles with FP32 or FP16 storage step H and E
 * in one launch, reported in [1] (and 0 in [2]).  The steps advance the simulation like
 * lx_sim_step. */
LX_API lx_status lx_sim_time_kernels(lx_sim* sim, int nsteps, double out_ms[4]);

/* Sizes of a handle's device state (engine feature). */
typedef struct lx_info {
  size_t cells;          /* Nx*Ny*Nz */
  size_t device_bytes;   /* device memory held by the handle now */
  size_t psi_h_entries;  /* stored CPML psi entries updated by the H kernel */
  size_t psi_e_entries;  /* ... by the E kernel */
  int slab[3];           /* stored psi depth per axis (0: no CPML on that axis) */
  int uniform;           /* 1 when dx = dy = dz (curls kept as plain differences) */
  int field_bytes;       /* bytes per stored field value (8, 4 or 2) */
} lx_info;
LX_API lx_status lx_sim_info(const lx_sim* sim, lx_info* info);

/* Counters since creation: device kernels launched, bytes copied host->device and
 * device->host by the handle. */
LX_API lx_status lx_sim_counters(const lx_sim* sim, uint64_t* kernels, uint64_t* h2d, uint64_t* d2h);

/* Page-locked host memory for fast transfers (cudaHostAlloc). */
LX_API lx_status lx_host_alloc(size_t bytes, void** ptr);
LX_API void lx_host_free(void* ptr);

LX_API const char* lx_last_error(const lx_sim* sim);
LX_API const char* lx_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LUXUM_H */
