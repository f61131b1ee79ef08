/*
 * lbgb300.h -- C ABI of the GB300 lattice Boltzmann library (liblbgb300.so).
 *
 * Part 1 are the reference's own entry points, with the reference's names,
 * argument order and meaning, so that the reference's host loop
 * (SimulationD2Q9/SimulationD3Q19::runLBM) links against this library
 * unchanged.  Each declaration names the reference interface it replaces.
 * Like the reference they return void; a failure is recorded and can be read
 * with lb_abi_last_error().  grid/block are accepted for signature
 * compatibility; the library picks its own launch shapes (and therefore does
 * not require width % 32 == 0 or height % 4 == 0).
 *
 * Part 2 is this library's own context API: one lattice per context, state
 * owned and laid out by the library, every call returns an lb_status.
 */
#ifndef LBGB300_H
#define LBGB300_H

#include <stdint.h>
#include "lattibol.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================== */
/* Part 1: drop-in entry points                                             */
/* ======================================================================== */

/* replaces streaming_d2q9, reference src/streaming.h:31-32 */
void streaming_d2q9(DataD2Q9 *data, dim3 grid, dim3 block);
/* replaces streaming_d3q19, reference src/streaming.h:34-35 */
void streaming_d3q19(DataD3Q19 *data, dim3 grid, dim3 block);

/* replaces collision_d2q9, reference src/collision.h:27-31 (includes the
 * Shan-Chen force step, reference src/collision.cu:352-354, when G < 0) */
void collision_d2q9(float *plot_data, DataD2Q9 *data, float w0, float w1, float w5,
                    float tau_inv, float ux_in, float uy_in, float rho_out, float u_min,
                    float u_max, float rho_min, float rho_max, dim3 grid, dim3 block,
                    float Fx, float Fy, float G, float Gads);
/* replaces collision_d3q19, reference src/collision.h:33-36 */
void collision_d3q19(float *plot_data, DataD3Q19 *data, float w0, float w1, float w7,
                     float tau_inv, float ux_in, float uy_in, float uz_in, float rho_out,
                     float u_min, float u_max, float rho_min, float rho_max, dim3 grid,
                     dim3 block);

/* replace get_border_d2q9/_d3q19, reference src/get_border.h:29-33 */
void get_border_d2q9(DataD2Q9 *data, dim3 grid, dim3 block);
void get_border_d3q19(DataD3Q19 *data, dim3 grid, dim3 block);
/* replace apply_border_d2q9/_d3q19, reference src/apply_border.h:25-29 */
void apply_border_d2q9(DataD2Q9 *data, dim3 grid, dim3 block);
void apply_border_d3q19(DataD3Q19 *data, dim3 grid, dim3 block);

/* replace read_value_2d/_3d, reference src/read_value.h:27-31.  plot_data may
 * be NULL (headless), then the probe reads the moment arrays instead. */
void read_value_2d(float *plot_data, DataD2Q9 *data, int x, int y, int z);
void read_value_3d(float *plot_data, DataD3Q19 *data, int x, int y, int z);

/* replaces copy_border_devices_d2q9, reference src/copy_border.h:30-35
 * (extern "C" there; the stream is passed by reference in C++) */
#ifdef __cplusplus
void copy_border_devices_d2q9(float *nb_border_f1, float *nb_border_f5, float *nb_border_f8,
                              float *nb_border_f3, float *nb_border_f6, float *nb_border_f7,
                              float *border_f1, float *border_f5, float *border_f8,
                              float *border_f3, float *border_f6, float *border_f7,
                              int height, cudaStream_t &s);
#else
void copy_border_devices_d2q9(float *nb_border_f1, float *nb_border_f5, float *nb_border_f8,
                              float *nb_border_f3, float *nb_border_f6, float *nb_border_f7,
                              float *border_f1, float *border_f5, float *border_f8,
                              float *border_f3, float *border_f6, float *border_f7,
                              int height, cudaStream_t *s);
#endif
/* C-linkage twin of copy_border_devices_d3q19, which the reference declares
 * with C++ linkage (reference src/copy_border.h:37-47); the library also
 * exports that C++ symbol itself.  dst[10]/src[10] are in the order
 * {f1, f7, f8, f9, f10, f2, f11, f12, f13, f14}. */
void lb_copy_border_devices_d3q19(float *const dst[10], float *const src[10], int height,
                                  int depth, cudaStream_t s);

/* --- drop-in controls (no counterpart in the reference) ------------------ */
#define LB_ABI_STANDALONE 0 /* streaming_* swaps in place, collision_* collides: the
                               reference's two-pass scheme, bit-identical results */
#define LB_ABI_FUSED 1      /* streaming_* records the step, collision_* runs one fused
                               pull-stream+collide into a library-owned second population
                               set and swaps the f* pointers inside *data */
int lb_abi_set_mode(int mode);
int lb_abi_get_mode(void);
/* fused mode: copy the current populations back into the caller's original
 * buffers, restore the caller's pointers in *data and free the second set */
int lb_abi_release_d2q9(DataD2Q9 *data);
int lb_abi_release_d3q19(DataD3Q19 *data);
/* global conservation sums over non-solid nodes, accumulated in FP64 on the
 * GPU from the moment arrays: out = {mass, mom_x, mom_y, mom_z, kinetic
 * energy, max|u|, n_fluid}.  Sums on the device current at the call, with
 * scratch kept per device (allocated by the first call on that device), so
 * the pointers in *data must be that device's.  Blocks the calling thread
 * until done. */
int lb_reduce_d2q9(const DataD2Q9 *data, double out[7]);
int lb_reduce_d3q19(const DataD3Q19 *data, double out[7]);
/* No counterpart in the reference.  The sums of lb_reduce_d3q19 for callers
 * that cannot allocate device memory (a host whose GPU memory all belongs to
 * its own pool allocator, or a real-time loop in which cudaMalloc/cudaFree
 * could synchronise the device).  It calls no allocator: its scratch is a
 * fixed 128 KiB array in the library's device memory, which every GPU that
 * loads the library keeps until the process exits.  Lattices of more than
 * 153 288 704 nodes are rejected with LB_ERR_ARG and a message in
 * lb_abi_last_error().  The first call on a device looks up the array's
 * device address.  Every call blocks the calling thread (it ends with a
 * synchronous copy of the 7 results to *out), so it must not be called while
 * a stream capture is in progress.  Calls share the array, so calls that
 * overlap on the GPU race; results equal lb_reduce_d3q19's up to FP64
 * summation order. */
int lb_reduce_d3q19_noalloc(const DataD3Q19 *data, double out[7]);
/* The reference's per-step host sequence (SimulationD3Q19::runLBM, reference
 * src/simulation_d3q19.cu:350-430, without the GL map/unmap and the extra
 * device-wide synchronisations): for each step streaming_d3q19,
 * collision_d3q19 into plot_data, read_value_3d's kernel at the cursor and
 * a 16-byte device-to-host copy of data->valueCur into value_host[4], all
 * queued in stream order (the host waits once, after the last step; the
 * value of the last step is left in value_host).  Returns LB_OK, LB_ERR_ARG
 * (bad struct or cursor outside the lattice) or LB_ERR_CUDA (message in
 * lb_abi_last_error). */
typedef struct {
    float w0, w1, w7, tau_inv, ux_in, uy_in, uz_in, rho_out;
    int cursor[3];
} lb_run_params_d3q19;
int lb_run_lbm_d3q19(DataD3Q19 *data, float *plot_data, const lb_run_params_d3q19 *p, int steps,
                     float *value_host);

/* last error recorded by a void drop-in call on this thread ("" if none) */
const char *lb_abi_last_error(void);
int lb_abi_clear_error(void);

/* ======================================================================== */
/* Part 2: context API                                                      */
/* ======================================================================== */

typedef enum {
    LB_OK = 0,
    LB_ERR_ARG = -1,     /* invalid argument or configuration */
    LB_ERR_CUDA = -2,    /* a CUDA call failed (message in lb_error) */
    LB_ERR_STATE = -3,   /* call not valid in the context's current state */
    LB_ERR_NOMEM = -4,   /* device allocation failed */
    LB_ERR_DEVICE = -5,  /* a kernel reported a device-side error (NaN census, bounds) */
    LB_ERR_IO = -6,      /* a file could not be opened, read or written, or its format
                            is not supported */
} lb_status;

#define LB_D2Q9 9
#define LB_D3Q19 19

#define LB_MODE_REFERENCE 0 /* reference semantics: walls stored as full-way bounce-back,
                               Zou-He inlet (x=0) and outlet (x=nx-1) always on */
#define LB_MODE_NATIVE 1    /* periodic box, half-way bounce-back at wall cells,
                               moving walls, body force, optional Shan-Chen */

#define LB_STORE_F32 0
#define LB_STORE_F16 1  /* populations stored as binary16 deviations f_k - w_k */
#define LB_STORE_BF16 2 /* populations stored as bfloat16 deviations f_k - w_k */

#define LB_PSI_REF 0    /* psi = 4 exp(-200/rho), the reference's form */
#define LB_PSI_EXP1 1   /* psi = 1 - exp(-rho) */

/* cell flags (lb_set_flags); in LB_MODE_REFERENCE any non-zero value is a
 * solid node */
#define LB_CELL_FLUID 0x00u
#define LB_CELL_WALL 0x01u
#define LB_CELL_MOVING 0x02u /* with LB_CELL_WALL: wall moving with config.wall_u */

/* launch tuning (lb_config.tuning); results do not depend on it */
#define LB_TUNE_DEFAULT 0      /* the library's measured choice */
#define LB_TUNE_EXPLICIT 0x100 /* use exactly the bits below */
#define LB_TUNE_PDL 0x008      /* D2Q9 without Shan-Chen: each step is a programmatic
                                  dependent launch of the previous one, so its launch
                                  overlaps the previous step's tail */
#define LB_TUNE_REVERSE 0x001  /* sweep the lattice in the opposite order on every
                                  other step, so a step starts where the previous
                                  one ended and its last writes are still in L2 */
#define LB_TUNE_TBLOCK 0x020   /* D2Q9 native mode without Shan-Chen: temporal
                                  blocking, one launch advances several steps of a
                                  tile and its halo in shared memory */
#define LB_TUNE_SC_STAGED 0x040 /* D3Q19 Shan-Chen on lattices without wall nodes
                                   (nx a multiple of 32, ny of 8, nz of 4): the
                                   single-pass step whose populations arrive in
                                   shared memory by asynchronous copies issued
                                   ahead of use; part of the default */
#define LB_TUNE_SC_NO_TMA 0x080 /* staged Shan-Chen step, 16-bit storage: copy
                                   every stage with 16-byte cp.async chunks, also
                                   where TMA tensor copies could (the interior
                                   tiles); same results (FP32 always uses cp.async) */
#define LB_TUNE_TBLOCK_SHAPE(n) ((n) << 12) /* with LB_TUNE_TBLOCK: block shape 1..10
                                               (steps per launch x tile), 0 = the
                                               library's choice */

typedef struct {
    int lattice;        /* LB_D2Q9 or LB_D3Q19 */
    int nx, ny, nz;     /* nodes; nz = 1 for D2Q9 */
    int mode;           /* LB_MODE_* */
    int storage;        /* LB_STORE_* */
    float tau_inv;      /* 1/tau */
    float force[3];     /* body force (velocity-shift forcing) */
    float u_in[3];      /* reference mode: inlet velocity (x used) */
    float rho_out;      /* reference mode: outlet density */
    float wall_u[3];    /* native mode: velocity of LB_CELL_MOVING walls */
    float G, G_ads;     /* Shan-Chen interaction and adhesion strengths (0 = off) */
    int psi_form;       /* LB_PSI_* */
    int graph_steps;    /* steps per captured CUDA graph in lb_step (0 = default 64) */
    int tuning;         /* LB_TUNE_* bits; LB_TUNE_DEFAULT picks the measured best */
    float rho_ref;      /* 16-bit storage keeps f_k - w_k*rho_ref (0 = 1.0) */
} lb_config;

typedef struct lb_ctx lb_ctx;

int lb_config_default(lb_config *cfg, int lattice, int nx, int ny, int nz);
int lb_create(const lb_config *cfg, lb_ctx **out);
int lb_destroy(lb_ctx *ctx);
const char *lb_error(const lb_ctx *ctx);

/* cell flags, one byte per node, host memory */
int lb_set_flags(lb_ctx *ctx, const uint8_t *flags);
/* populations in the library's SoA order f[k*N + node], host float memory */
int lb_set_populations(lb_ctx *ctx, const float *f);
int lb_get_populations(lb_ctx *ctx, float *f);
/* equilibrium from host moment fields (any of ux/uy/uz may be NULL = 0; rho
 * NULL = 1) */
int lb_init_equilibrium(lb_ctx *ctx, const float *rho, const float *ux, const float *uy,
                        const float *uz);
/* advance nsteps time steps (asynchronous on the context's stream); the
 * moments of the last step are written to the moment fields */
int lb_step(lb_ctx *ctx, int nsteps);
/* the moment fields of the last step (host memory; uz ignored for D2Q9) */
int lb_get_moments(lb_ctx *ctx, float *rho, float *ux, float *uy, float *uz);
/* conservation sums of the last step's moments, FP64 (see lb_reduce_d3q19) */
int lb_reduce(lb_ctx *ctx, double out[7]);
/* (ux, uy, uz, rho) of the last step at one node, copied to host memory
 * (blocks until the copy is done) -- the context form of read_value_3d */
int lb_probe(lb_ctx *ctx, int x, int y, int z, float value[4]);
/* the reference's per-step host pattern on a context (a step, then the
 * cursor value read to the host): every step's kernel writes (ux, uy, uz, rho)
 * of node (x, y, z) into mapped page-locked host memory, so the steps replay
 * from graphs without a host round trip between them; value[4] holds the last
 * step's, the moment fields the last step's.  (The closure and single-pass
 * Shan-Chen kernels fall back to a step plus lb_probe per step.) */
int lb_run_probe(lb_ctx *ctx, int nsteps, int x, int y, int z, float value[4]);
int lb_synchronize(lb_ctx *ctx);
/* run nsteps and return the device time between CUDA events recorded on the
 * context's stream (warm-up is the caller's business) */
int lb_time_steps(lb_ctx *ctx, int nsteps, float *ms);
/* number of kernel launches issued by this context so far */
int64_t lb_launch_count(const lb_ctx *ctx);
/* the moving-wall momentum term 6 w_k (c_k . wall_u) per direction, as used
 * by the kernels (q = 9 or 19 floats) */
int lb_wall_correction(const lb_ctx *ctx, float *corr);

/* ======================================================================== */
/* Part 3: ensembles of independent periodic D2Q9 Shan-Chen domains        */
/* ======================================================================== */
/* Many small lattices of different sizes advanced together: one packed
 * population slab (domain d at nodes [offset(d), offset(d) + nx[d]*ny[d]),
 * node x + nx[d]*y inside it), two persistent launches per step over a work
 * list of row groups, batches replayed from a captured CUDA graph.  Each
 * domain is periodic, without walls or body force, with its own G and
 * tau_inv; a domain evolves bit for bit like the same lattice run alone
 * through the context API (native mode, same psi form). */
typedef struct lb_ensemble lb_ensemble;
int lb_ensemble_create(int ndomains, const int *nx, const int *ny, const float *G,
                       const float *tau_inv, int psi_form, lb_ensemble **out);
int lb_ensemble_destroy(lb_ensemble *e);
const char *lb_ensemble_error(const lb_ensemble *e);
long lb_ensemble_nodes(const lb_ensemble *e);          /* total nodes of all domains */
long lb_ensemble_offset(const lb_ensemble *e, int d);  /* first node of domain d */
/* populations f[k*nodes + node] / equilibrium at u = 0 from a packed density */
int lb_ensemble_set_populations(lb_ensemble *e, const float *f);
int lb_ensemble_get_populations(lb_ensemble *e, float *f);
int lb_ensemble_init_equilibrium(lb_ensemble *e, const float *rho);
int lb_ensemble_step(lb_ensemble *e, int nsteps);  /* last step writes the moments */
int lb_ensemble_time_steps(lb_ensemble *e, int nsteps, float *ms);
int lb_ensemble_get_moments(lb_ensemble *e, float *rho, float *ux, float *uy);
/* launch shape.  threads_x = 0: one launch per step; rows then picks the
 * form: 1..5 tiles that form psi of the tile and its ring in shared memory
 * (1: 32 x 8 at 48 registers; 2: 32 x 8 at 40; 3: 32 x 16 at 60; 4: 32 x 16
 * at 40; 5: 32 x 32 at 60), 6..9 warps marching down 32-column strips with
 * psi of three rows in registers (6: 32 rows at 80 registers; 7: 32 rows at
 * 64; 8: 64 rows; 9: 16 rows), 10..12 the same strips fed by a per-warp
 * shared-memory ring of source rows copied ahead with cp.async (10: 32 rows,
 * the default with 3 blocks per SM; 11: 64 rows; 12: 16 rows; domains not a
 * multiple of 32 wide, or not starting on a 16-byte boundary, take the plain
 * strips).  Otherwise the two-pass step (psi pass, fused pass)
 * over groups of `rows` rows with threads_x threads along x (a multiple of
 * 32).  Both give the same bits.  The autotuner times every candidate for
 * trial_steps steps on the ensemble itself (advancing its state: tune before
 * initialising) and keeps the fastest, returned in out[3] */
int lb_ensemble_set_launch(lb_ensemble *e, int threads_x, int rows, int blocks_per_sm);
int lb_ensemble_get_launch(const lb_ensemble *e, int out[3]);
int lb_ensemble_autotune(lb_ensemble *e, int trial_steps, int out[3]);
int64_t lb_ensemble_launch_count(const lb_ensemble *e);

/* ======================================================================== */
/* Part 4: learned sub-grid closure (D3Q19)                                 */
/* ======================================================================== */
/* A 19 -> 64 -> 64 -> 1 ReLU network maps each cell's non-equilibrium
 * moments and |S| to an eddy viscosity nu_t = nu0 * clamp(y, 0, z_max); the
 * closure kernel relaxes the cell with tau = 0.5 + 3 (nu0 + nu_t).  The
 * network runs on the tcgen05 tensor cores (BF16 weights and activations,
 * FP32 accumulators in tensor memory) inside the collision kernel; training
 * runs its forward and backward passes on the tensor cores the same way
 * (the gradient contractions' operands in BF16, FP32 accumulation) and Adam,
 * all on the GPU.  Every tensor-core wait is bounded: a network call whose
 * MMA never completed returns LB_ERR_CUDA (lb_mlp_error says so). */
typedef struct lb_mlp lb_mlp;
int lb_mlp_create(uint64_t seed, lb_mlp **out);  /* He-uniform initial weights */
int lb_mlp_destroy(lb_mlp *m);
const char *lb_mlp_error(const lb_mlp *m);
int lb_mlp_num_params(void);  /* 5505: W1[64][19], b1, W2[64][64], b2, w3[64], b3 */
int lb_mlp_set_params(lb_mlp *m, const float *params);  /* resets the Adam state */
int lb_mlp_get_params(lb_mlp *m, float *params);
/* network outputs y[n] for device rows x_dev[n][19] (the closure's forward) */
int lb_mlp_forward(lb_mlp *m, const float *x_dev, float *y_dev, long n);
/* gradient (host, 5505 floats) and value of the mean squared error over all n
 * device samples */
int lb_mlp_grad(lb_mlp *m, const float *x_dev, const float *z_dev, long n, float *grad,
                double *loss);
/* Adam (beta 0.9/0.999) for `steps` minibatches of `batch` contiguous samples
 * starting at seeded random offsets; loss_log[steps] optional (host) */
int lb_mlp_train(lb_mlp *m, const float *x_dev, const float *z_dev, long n, int steps,
                 int batch, float lr, uint64_t seed, float *loss_log);
/* install the closure on a D3Q19 native FP32 context (m == NULL removes it);
 * the network must outlive its use; its biases and output layer are read at
 * this call (call it again after further training); y_out_dev (optional, N
 * floats) receives the raw network output of every fluid cell at each step */
int lb_closure_enable(lb_ctx *ctx, const lb_mlp *m, float nu0, float s_ref, float z_max,
                      float *y_out_dev);
/* training data from a fine lattice's last-step moment fields: Favre box
 * filter by `factor`, features [Nc][19] and targets z = nu_t/nu0 [Nc]
 * (device buffers; NULL to skip) and the mean resolved kinetic energy of the
 * filtered field */
int lb_closure_sample(lb_ctx *fine, int factor, float nu0, float s_ref, float z_max,
                      float *features_dev, float *targets_dev, double *ke_mean);
/* the same with the target's two contractions T_dev : S and S : S summed over
 * the (2 avg_radius + 1)^3 coarse cells around each cell (periodic) before
 * nu_t = max(0, -sum(T_dev : S) / (2 sum(S : S))) is formed (avg_radius 0 is
 * lb_closure_sample) */
int lb_closure_sample_avg(lb_ctx *fine, int factor, float nu0, float s_ref, float z_max,
                          int avg_radius, float *features_dev, float *targets_dev,
                          double *ke_mean);
/* device pointers of a context's moment fields (valid until lb_destroy) and
 * its extents */
int lb_device_fields(lb_ctx *ctx, float **rho, float **ux, float **uy, float **uz);
/* self-check of the tensor-core (tcgen05) pattern the closure kernel uses, in
 * one CTA, three rounds: out[round][0] (128 x 64) = X W1^T with
 * X[r][k] = ((7r + 3k) mod 9 - 4)(round + 1), W1[n][k] = (5n + k) mod 7 - 3,
 * k < 32; out[round][1] = H W2^T with H[r][k] = (r + 3k + round) mod 5 - 2,
 * W2[n][k] = (n + 2k) mod 5 - 2, k < 64 (exact small integers).  *status
 * gets bit 2i (bit 2i+1) when round i's first (second) MMA never completed. */
int lb_tcgen05_selftest(float *out, int *status);
/* self-check of the bounded waits on the GPU: which = 1 makes the tcgen05
 * kernels' mbarrier wait run out (nothing committed), which = 2 the staged
 * Shan-Chen step's stage wait (given no polls; the block then waits for the
 * copies it issued before it returns).  *status = 1 when the wait gave up as
 * designed, reported the failure and returned. */
int lb_wait_selftest(int which, int *status);
int lb_extents(const lb_ctx *ctx, int *nx, int *ny, int *nz);

/* ======================================================================== */
/* Part 5: case files -- the reference's Input class (src/input.cpp) and    */
/* the initial state its Simulation constructors build                      */
/* ======================================================================== */

/* Functions without a context report failures through lb_abi_last_error(). */

/* the parameter file (.dat), one value per line, read as reference
 * src/input.cpp:51-94 (Input::loadParameters) reads it: a missing line or one
 * that is not a number reads as 0; lines after the 13th are ignored */
typedef struct {
    int device_count;   /* line 1 */
    int max_dim;        /* line 2; <= 1 means a 2-D case (stored as 1) */
    float ux, uy, uz;   /* lines 3-5: inlet and initial velocity */
    float rho;          /* line 6: outlet and initial density */
    float viscosity;    /* line 7 */
    int update_steps;   /* line 8: steps between two display updates */
    float ext_f[3];     /* lines 9-11: body force (Fx, Fy, Fz) */
    float G;            /* line 12: Shan-Chen interaction strength */
    float G_ads;        /* line 13: fluid-solid adhesion strength */
    float tau_inv;      /* 1 / (3 viscosity + 0.5), src/input.cpp:168-171 */
    float min_u, max_u, min_rho, max_rho; /* colour scales, src/input.cpp:88-91 */
} lb_case_params;

/* reference src/input.cpp:51-94; LB_ERR_IO when the file cannot be opened */
int lb_case_load_parameters(const char *path, lb_case_params *out);

/* The solid mask of a 2-D case from a Windows bitmap, as reference
 * src/input.cpp:96-116 (Input::loadSolids): a node is solid where the pixel
 * is opaque black, solids[x + y*width] with y = 0 the top row of the image.
 * Supported: uncompressed 1/4/8/16/24/32 bits per pixel and BI_BITFIELDS
 * 16/32, bottom-up or top-down.  Call with solids = NULL to read the size;
 * capacity is the size of solids in bytes. */
int lb_case_load_solids_bmp(const char *path, int *width, int *height, uint8_t *solids,
                            size_t capacity);

/* Triangles of a binary or ASCII STL file, 9 floats each (three vertices);
 * call with tri = NULL for the count.  capacity is in floats. */
int lb_stl_read(const char *path, int64_t *ntri, float *tri, size_t capacity);
/* The solid mask of a closed triangle surface on the GPU (the stand-in for
 * the reference's cvmlcpp voxelisation in Input::loadSolidsSTL,
 * src/input.cpp:118-142, which is not part of the reference tree): the
 * longest bounding-box side spans max_dim voxels, each axis
 * ceil(extent / voxel) voxels (dims = W, H, D); a voxel is solid when its
 * centre is inside the surface (crossing parity along z, fixed-point edge
 * functions with a consistent tie rule).  solids = NULL: dims only.
 * *open_columns (may be NULL) is set to 1 when some column crossed the
 * surface an odd number of times (an open surface). */
int lb_voxelize(const float *tri, int64_t ntri, int max_dim, int dims[3], uint8_t *solids,
                size_t capacity, int *open_columns);
/* lb_stl_read + lb_voxelize: Input::loadSolidsSTL of a 3-D case */
int lb_case_load_solids_stl(const char *path, int max_dim, int *width, int *height, int *depth,
                            uint8_t *solids, size_t capacity);

/* The initial D2Q9 state of reference src/simulation_d2q9.cu:100-334 for one
 * device over the whole width, in host memory: f is 9 arrays of
 * width*height floats (f[k*N + node]), the other outputs N values each
 * (psi, ueq_x, ueq_y may be NULL).  Values the reference leaves unset
 * (solid nodes of a Shan-Chen case) are 0, as fresh pages of the reference's
 * allocations are. */
int lb_case_init_d2q9(const lb_case_params *p, int width, int height, const uint8_t *solids,
                      float *f, float *ux, float *uy, float *rho, float *psi, float *ueq_x,
                      float *ueq_y, uint8_t *solid_bound);

/* The initial D3Q19 state of reference src/simulation_d3q19.cu:99-204 (one
 * device): uniform equilibrium at (ux, uy, uz, rho) and the solid_bound rule.
 * Like the reference it sets uz only at node 0 (uz[i > 0] = 0). */
int lb_case_init_d3q19(const lb_case_params *p, int width, int height, int depth,
                       const uint8_t *solids, float *f, float *ux, float *uy, float *uz,
                       float *rho, uint8_t *solid_bound);

/* ======================================================================== */
/* Part 6: output files and checkpoints                                     */
/* ======================================================================== */

/* The VTK image file "<dir>/rIIIIpDD.vti" of reference src/output.cpp:96-155
 * (Output::saveVTK): ASCII, "Pressure" = rho, "Velocity" = (ux, uy, uz) in
 * 3-D and (ux, -uy, 0) in 2-D (length == 1), x extent width+1 points with
 * a 0 closing every row.  vtk_id 0..9999, device_id 0..99; uz may be NULL in
 * 2-D. */
int lb_vtk_save(const char *dir, int vtk_id, int device_id, int width, int height, int length,
                const float *rho, const float *ux, const float *uy, const float *uz);
/* the parallel index "<dir>/rIIII.pvti" of reference src/output.cpp:52-94
 * (Output::saveParVTK) naming device_count pieces of width nodes each */
int lb_vtk_save_parallel(const char *dir, int vtk_id, int device_count, int width, int height,
                         int length);
/* the moments of a context's last step as a VTK file (device 0 of 1) */
int lb_vtk_save_ctx(lb_ctx *ctx, const char *dir, int vtk_id);

/* Checkpoints of a context: configuration, step count, cell flags, the
 * populations in their stored type (16-bit storage is saved as stored, so a
 * resumed run is bit-identical to an uninterrupted one) and the moment
 * fields, each section with a CRC-32.  The file is written beside the target
 * and renamed over it when complete. */
int lb_checkpoint_save(lb_ctx *ctx, const char *path);
/* restore into a context created with the same lattice, extents, mode and
 * storage (LB_ERR_ARG otherwise; LB_ERR_IO for a damaged file) */
int lb_checkpoint_load(lb_ctx *ctx, const char *path);
/* a new context with the checkpoint's configuration and state */
int lb_checkpoint_create(const char *path, lb_ctx **out);
/* the configuration and step count stored in a checkpoint */
int lb_checkpoint_info(const char *path, lb_config *cfg, int64_t *steps);
/* time steps a context has advanced since lb_create (restored by
 * lb_checkpoint_load) */
int64_t lb_steps_done(const lb_ctx *ctx);

/* ======================================================================== */
/* Part 7: z-slab decomposition (several devices or processes, one lattice) */
/* ======================================================================== */
/* Replaces the reference's x-slab halo exchange between devices:
 * get_border_d3q19 (src/get_border.cu:59-98) packs a face, copy_border_devices
 * (src/copy_border.cu:49-81) moves it to the neighbour, apply_border_d3q19
 * (src/apply_border.cu:58-97) unpacks it, driven once per step from
 * src/simulation_d3q19.cu:363-406.  Here the lattice is cut along z, the
 * slowest axis, so each of the 5 populations that cross a face is one
 * contiguous plane: lb_slab_step packs them (get_border), the caller or
 * lb_slab_group_step moves them (copy_border) and lb_slab_unpack writes them
 * into the receiving slab's ghost plane (apply_border).  The planes of the
 * step that the exchange does not need run on a second stream meanwhile.
 *
 * A slab context holds global planes z0 .. z0 + nz - 1 of a D3Q19 native-mode
 * lattice without Shan-Chen (global config *global, periodic in z) plus one
 * ghost plane below and one above, so every per-node array it takes or gives
 * (lb_set_flags, lb_set_populations, lb_get_populations, lb_init_equilibrium,
 * lb_get_moments) covers nz + 2 planes: global planes z0 - 1 .. z0 + nz, z
 * wrapped.  Flags must be given for the ghost planes too.  Moments of the
 * ghost planes are not computed; lb_reduce sums the own planes.  lb_step,
 * lb_run_probe, checkpoints and the closure are not available on a slab.
 *
 * Step protocol, per time step, with the face buffers on the slab's device
 * (face_bytes each = 5 nx ny stored values, [5][nx*ny], populations 6, 10, 14,
 * 16, 18 for the lower face and 5, 9, 13, 15, 17 for the upper one):
 *   lb_slab_step(ctx, moments, to_below, to_above);   - queues the step and
 *        the new faces on lb_stream(ctx)
 *   (transport on lb_stream(ctx): to_below -> the lower neighbour's from_above,
 *    to_above -> the upper neighbour's from_below)
 *   lb_slab_unpack(ctx, from_below, from_above);     - ghost planes of the new state
 * Before the first step the ghost planes hold what lb_set_populations or
 * lb_init_equilibrium gave them; lb_slab_pack gives the current faces (to
 * refresh the ghosts of a state set some other way).  Results are bit-identical
 * to the same steps of one context over the whole lattice. */
int lb_slab_create(const lb_config *global, int z0, int nz, lb_ctx **out);
int lb_slab_info(const lb_ctx *ctx, int *z0, int *nz, int *nz_global, size_t *face_bytes);
/* the context's CUDA stream (cudaStream_t) for an external transport */
void *lb_stream(lb_ctx *ctx);
int lb_slab_pack(lb_ctx *ctx, void *to_below, void *to_above);
int lb_slab_step(lb_ctx *ctx, int moments, void *to_below, void *to_above);
int lb_slab_unpack(lb_ctx *ctx, const void *from_below, const void *from_above);
/* nsteps steps of all n slabs of one lattice held by this process on the
 * current device (slabs[i] the z-neighbour above slabs[i-1], periodic), the
 * faces moved by device copies; the last step writes the moments.
 * Asynchronous (lb_synchronize each slab). */
int lb_slab_group_step(lb_ctx *const *slabs, int n, int nsteps);
/* lb_slab_group_step timed on the device: *ms from an event before any slab's
 * first launch to one after every slab's last (blocks until done) */
int lb_slab_group_time(lb_ctx *const *slabs, int n, int nsteps, float *ms);

/* ---- device helpers (tests and hosts without their own allocator) ------ */
int lb_device_count(int *n);
/* the device this thread's later calls (lb_create, lb_slab_create, ...) use;
 * one process per GPU selects its own (its local rank) before creating any
 * context */
int lb_set_device(int dev);
int lb_malloc(void **ptr, size_t bytes);
int lb_free(void *ptr);
int lb_malloc_host(void **ptr, size_t bytes); /* page-locked host memory */
int lb_free_host(void *ptr);
int lb_memcpy_h2d(void *dst, const void *src, size_t bytes);
int lb_memcpy_d2h(void *dst, const void *src, size_t bytes);
int lb_memset(void *dst, int value, size_t bytes);
int lb_device_synchronize(void);
const char *lb_version(void);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
/* the reference's C++-linkage entry point, reference src/copy_border.h:37-47 */
void copy_border_devices_d3q19(float *nb_border_f1, float *nb_border_f7, float *nb_border_f8,
                               float *nb_border_f9, float *nb_border_f10, float *nb_border_f2,
                               float *nb_border_f11, float *nb_border_f12,
                               float *nb_border_f13, float *nb_border_f14, float *border_f1,
                               float *border_f7, float *border_f8, float *border_f9,
                               float *border_f10, float *border_f2, float *border_f11,
                               float *border_f12, float *border_f13, float *border_f14,
                               int height, int depth, cudaStream_t &s);
#endif

#endif
