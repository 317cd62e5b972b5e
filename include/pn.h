/*
 * pn.h -- C ABI of libpn: the Limit-sticky9 direct-summation force path on one GB300 (sm_103a).
 *
 * Three layers, all plain C types (no CUDA or torch types in any signature):
 *
 *  1. Drop-in entry points with the reference's own names and signatures, so the reference's
 *     main loop (Limit-sticky9.c:740-920) links against this library unchanged:
 *       force            replaces Limit-sticky9.c:21-424
 *       energy           replaces Limit-sticky9.c:427-564  (prints the same three lines)
 *       initial_energy   replaces Limit-sticky9.c:566-714  (prints the same two lines)
 *       push_velocity / push_position   replace Limit-sticky9.c:716-738 (host loops, unused
 *                                        by the reference main; kept for link compatibility)
 *     Arrays are the caller's host AoS arrays double[n][3] with index 0 = the black hole (BH),
 *     exactly as in the reference.  Each call copies x, v, m to the GPU and the result back,
 *     as the Goose-generated GPU variant did.  Errors: these keep the reference's void
 *     signatures; pn_last_error() reports the last status, and a CUDA failure aborts with a
 *     message (the Goose variant called exit(1), Limit-sticky9_nvidia.cu:89-114).
 *
 *  2. A device-resident context (pn_ctx) that keeps the state on the GPU between force
 *     evaluations and runs whole integration steps (the reference's 3-evaluation
 *     Runge-Kutta step, Limit-sticky9.c:841-893) as one CUDA graph per step.
 *
 *  3. Host utilities: initial-condition generators and the reference's text formats
 *     (input Limit-sticky9.c:796-809, snapshots :820-826 / :899-905).
 *
 * Units are G = 1; the 1PN terms are weighted by inv_c2 (1.0 reproduces the reference,
 * which has c = 1 implicitly; 0.0 gives the Newtonian force alone).  All functions returning
 * int return PN_OK (0) or a negative pn_status.
 */
#ifndef PN_H
#define PN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PN_NMAX 270000 /* Limit-sticky9.c:13: the drop-in entry points accept n <= PN_NMAX */

typedef enum {
    PN_OK = 0,
    PN_ERR_INVALID = -1,     /* bad argument (n out of range, NULL pointer, eps <= 0, ...) */
    PN_ERR_CUDA = -2,        /* a CUDA runtime call failed */
    PN_ERR_NOMEM = -3,       /* device or host allocation failed */
    PN_ERR_NONFINITE = -4,   /* a force or energy came out NaN/Inf */
    PN_ERR_IO = -5,          /* file open/parse error */
    PN_ERR_TIMEOUT = -6,     /* a bounded in-kernel wait gave up (the kernel returned early) */
    PN_ERR_UNSUPPORTED = -7, /* no GPU, or a configuration this build does not support */
    PN_ERR_STATE = -8        /* call out of order (e.g. no state set) */
} pn_status;

typedef enum {
    PN_PREC_FP64 = 0,  /* every pair term in FP64: parity with the reference */
    PN_PREC_MIXED = 1  /* FP32 pair terms (per-tile FP64 origin, compensated sums), FP64 rest */
} pn_precision;

typedef struct {
    double eps;        /* Plummer softening (Limit-sticky9.c:770) */
    double dt;         /* time step (Limit-sticky9.c:771) */
    double inv_c2;     /* weight of the 1PN terms; 1.0 = reference */
    int precision;     /* pn_precision */
    int tile_j;        /* j-particles per shared-memory tile; 0 = tuned */
    int i_per_thread;  /* i-particles held per thread; 0 = tuned */
    int j_split;       /* lanes sharing one i-set (warp-shuffle reduction); 0 = tuned */
    int grid_split;    /* CTAs sharing one i-block (partial sums reduced in FP64); 0 = tuned */
    int pair_variant;  /* mixed mode: PN_PAIR_AUTO (0, tuned), PN_PAIR_SCALAR (1),
                          PN_PAIR_F32X2 (2: packed FP32x2 instructions, two j per instruction) or
                          PN_PAIR_F32X2_OCC3 (3: the same with 2 i per thread, compiled for 3
                          CTAs per SM) or PN_PAIR_F32X2_OCC4 (4: ... for 4 CTAs per SM) */
    int integrator;    /* PN_INT_REFERENCE (0): the reference's 3-evaluation scheme
                          (Limit-sticky9.c:844-893); PN_INT_RK4 (1): classic 4th-order RK */
} pn_params;

enum { PN_PAIR_AUTO = 0, PN_PAIR_SCALAR = 1, PN_PAIR_F32X2 = 2, PN_PAIR_F32X2_OCC3 = 3, PN_PAIR_F32X2_OCC4 = 4 };
enum { PN_INT_REFERENCE = 0, PN_INT_RK4 = 1 };

/* Energies as the reference prints them (Limit-sticky9.c:561-562, :702-703). */
typedef struct {
    double pot_n;  /* Newtonian potential energy */
    double kin_n;  /* Newtonian kinetic energy */
    double pot_pn; /* O(N) 1PN BH-star energy */
    double total;  /* kin_n + pot_n + pot_pn + sum of the pairwise 1PN energy */
} pn_energy_t;

/* Kernel timing/accounting of the last device operation (for benchmarks). */
typedef struct {
    double pair_ms;          /* time of the last O(N^2) pair kernel launch (CUDA events) */
    double total_ms;         /* whole force evaluation */
    double interactions;     /* star-star pairs evaluated by that launch */
    int tile_j, i_per_thread, j_split, grid_split, threads; /* launch shape used */
    int pair_variant;        /* PN_PAIR_SCALAR, PN_PAIR_F32X2, _OCC3 or _OCC4: the kernel used */
} pn_stats;

/* ------------------------------------------------------------------ 1. drop-in entry points */
void force(double (*x)[3], double (*v)[3], double *m, double eps, double (*a)[3], double *pot,
           int n);
void energy(double t, double x[][3], double v[][3], double m[], int n, double init_ene,
            double eps);
void initial_energy(double x[][3], double v[][3], double m[], int n, double *init_ene,
                    double eps);
void push_velocity(double v[][3], double a[][3], double dt, int n);
void push_position(double x[][3], double v[][3], double dt, int n);

/* Status of the last drop-in call on this thread (PN_OK after a successful one). */
int pn_last_error(void);
/* Human-readable detail of the last error on this thread ("" when none). */
const char *pn_last_error_message(void);
const char *pn_strerror(int status);
/* Precision of the drop-in entry points (default PN_PREC_FP64; the environment variable
 * PN_PRECISION=mixed selects PN_PREC_MIXED at first use).  Also sets inv_c2 for them. */
int pn_dropin_configure(int precision, double inv_c2);
/* Releases the drop-in entry points' implicit context (optional; also done at exit). */
void pn_dropin_release(void);

/* ------------------------------------------------------------------ 2. device-resident API */
typedef struct pn_ctx pn_ctx;

void pn_params_default(pn_params *p);
/* Creates a context for up to nmax particles (BH included) on the current CUDA device. */
int pn_create(pn_ctx **ctx, int nmax, const pn_params *p);
int pn_destroy(pn_ctx *ctx);
/* Host AoS [n][3] state in / out (index 0 = BH). */
int pn_set_state(pn_ctx *ctx, int n, const double *x, const double *v, const double *m);
int pn_get_state(pn_ctx *ctx, double *x, double *v);
/* Acceleration at the current state into host AoS a[n][3] (one force() evaluation). */
int pn_force(pn_ctx *ctx, double *a);
/* nsteps integration steps of the reference's scheme (Limit-sticky9.c:844-893) on the
 * device-resident state; time advances by dt per step.  Asynchronous on the context's
 * stream: pn_sync() waits and returns the status of in-kernel checks. */
int pn_steps(pn_ctx *ctx, int nsteps);
int pn_sync(pn_ctx *ctx);
/* Energies of the current state (Limit-sticky9.c:445-556 arithmetic). */
int pn_energy(pn_ctx *ctx, pn_energy_t *e);
/* The energies of the current state, as pn_energy, and then nsteps (>= 1) integration steps,
 * as pn_steps: the energy's pair sums are accumulated by the first step's first force sweep,
 * which runs at that same state, so a snapshot's energy costs no sweep of its own (the
 * reference's main loop evaluates initial_energy() or energy() and then force() at the same
 * state, Limit-sticky9.c:837 or :896, then :851).  Waits for the steps, like pn_sync. */
int pn_steps_energy(pn_ctx *ctx, int nsteps, pn_energy_t *e);
/* pn_steps_energy in two halves: the first queues the steps and returns at once (like
 * pn_steps), the second waits for them and returns the energies of the state they started
 * from.  No other energy evaluation on the context may come in between. */
int pn_steps_energy_async(pn_ctx *ctx, int nsteps);
int pn_energy_result(pn_ctx *ctx, pn_energy_t *e);
/* A snapshot of the current state that does not stop the GPU: pn_snapshot_begin queues a copy
 * of x, v on the context's stream and its transfer to pinned host memory on a second stream, so
 * steps queued after it run while the transfer goes out; pn_snapshot_end waits for the transfer
 * only and writes host AoS x, v ([n][3]; either may be NULL).  One snapshot at a time. */
int pn_snapshot_begin(pn_ctx *ctx);
int pn_snapshot_end(pn_ctx *ctx, double *x, double *v);
double pn_time(pn_ctx *ctx);
int pn_get_stats(pn_ctx *ctx, pn_stats *s);
/* Changes the run parameters of an existing context (e.g. precision). */
int pn_set_params(pn_ctx *ctx, const pn_params *p);

/* Binary checkpoint of a context (state, masses, time, parameters) plus the calling loop's snapshot
 * clock and initial energy; pn_load_checkpoint restores all of it into an existing context
 * (n must fit its capacity).  Format: "PNCK0001", int32 n, doubles time, eouttime, init_ene,
 * the pn_params struct, then x, v (AoS [n][3]) and m [n], little-endian. */
int pn_save_checkpoint(pn_ctx *ctx, const char *path, double eouttime, double init_ene);
int pn_load_checkpoint(pn_ctx *ctx, const char *path, double *eouttime, double *init_ene);

/* Device-pointer entry point: one force evaluation on caller-owned device AoS arrays
 * (d_x, d_v: double[n][3]; d_m: double[n]; d_a: double[n][3] out) on the given stream
 * (a cudaStream_t passed as void*; NULL = the context's stream). */
int pn_force_device(pn_ctx *ctx, int n, const double *d_x, const double *d_v,
                    const double *d_m, double *d_a, void *stream);

/* Launch-shape autotuner.  Times candidate shapes of the pair sweep on the context's current
 * state (sweeps: bit 0 = the force sweep, bit 1 = the energy sweep) and keeps the fastest per
 * (precision, sweep, size class floor(log2 N)) for every context of this process; with the
 * environment variable PN_TUNE_CACHE=<file> the table is also kept in that file.  Shapes set
 * explicitly in pn_params take precedence.  best_ms (optional, [2]) gets the winning times. */
int pn_autotune(pn_ctx *ctx, int sweeps, double *best_ms);
void pn_autotune_clear(void);

/* Benchmark support.  Runs nsteps captured integration steps one at a time on the context's
 * stream; before each, optionally overwrites a buffer twice the size of L2 (flush_l2 != 0).
 * step_ms[k]: CUDA-event time of step k; pair_ms[k]: summed time of its three pair-sweep
 * launches (events captured in the step graph around each launch). */
int pn_bench_steps(pn_ctx *ctx, int nsteps, int flush_l2, double *step_ms, double *pair_ms);
/* Flops of one pair interaction of a sweep (mode 0 Newtonian, 1 force with 1PN, 2 energy) in
 * the given precision and pair variant (PN_PAIR_F32X2: the packed FP32x2 form, else the scalar
 * form); an FMA counts 2, the MUFU rsqrt 1, any other add or multiply 1. */
double pn_flops_per_pair(int mode, int precision, int pair_variant);
/* Measured FMA throughput of this GPU (TFLOP/s, FMA = 2 flops) in FP32 (PN_PREC_MIXED), FP64
 * (PN_PREC_FP64) or FP32 issued as the packed two-lane fma.rn.f32x2 that the packed sweep uses
 * (PN_PROBE_F32X2): the roofline denominators of the pair sweeps. */
enum { PN_PROBE_F32X2 = 2 };
int pn_probe_fma_peak(int precision, double *tflops);

/* Self-test of the in-kernel bounded waits: launches a kernel whose mbarrier wait can only end
 * by its time limit (about `seconds`, at most 5); returns PN_ERR_TIMEOUT when the limit
 * worked and the kernel returned on its own.  Faults nothing; the context stays usable. */
int pn_selftest_wait_timeout(pn_ctx *ctx, double seconds);

/* A force evaluation that allocates nothing.  No counterpart in the reference (its force()
 * allocates a 6.5 MB stack array per call).  For callers that cannot call cudaMalloc when they
 * need a force: a framework that owns all device memory through its own pool, a time-critical
 * loop in which cudaMalloc/cudaFree would stall the device, a plug-in host that forbids
 * allocation after start-up.  The caller passes device arrays d_x, d_v (AoS double[n][3]),
 * d_m (double[n]) and the output d_a (double[n][3]); precision is PN_PREC_FP64 or
 * PN_PREC_MIXED; stream is a cudaStream_t (NULL = the default stream) and the call is
 * asynchronous on it.  All work buffers live in one fixed device array of
 * PN_NOALLOC_SCRATCH_BYTES inside the library, held by every GPU that loads it until the
 * process exits, so n may not exceed PN_NOALLOC_NMAX (PN_ERR_INVALID otherwise).  The first call
 * on a device looks up that array's device address and the device's SM count (make it before
 * any stream capture).  Calls share the array: calls that overlap on the GPU race.  The return
 * value covers the host-side checks and the launches; what only the GPU can see (a non-finite
 * force, e.g. a star exactly on the BH; an in-kernel wait that gave up) is recorded in the
 * array's error word and read back by pn_noalloc_status. */
#define PN_NOALLOC_NMAX 8192
#define PN_NOALLOC_SCRATCH_BYTES 3364096
int pn_force_noalloc(int n, const double *d_x, const double *d_v, const double *d_m, double eps,
                     double inv_c2, int precision, double *d_a, void *stream);
/* Host-side status of the calling thread's last pn_force_noalloc call. */
int pn_noalloc_last_error(void);
/* Device-side status of the last pn_force_noalloc call on the current device: waits for
 * `stream` (the stream that call ran on), then copies the 4-byte error word into a host
 * variable (no allocation).  PN_OK, PN_ERR_NONFINITE or PN_ERR_TIMEOUT. */
int pn_noalloc_status(void *stream);

/* ------------------------------------------------------------------ 2a. discrete adjoint */
/* Vector-Jacobian product of one force evaluation at the current state: for abar (host AoS
 * [n][3], the adjoint of the accelerations) returns xbar = (da/dx)^T abar, vbar = (da/dv)^T
 * abar (host AoS [n][3]) and m0bar = abar . da/dm0 (the BH mass).  Same precision as the
 * context (FP64, or FP32 pair terms in mixed mode). */
int pn_force_vjp(pn_ctx *ctx, const double *abar, double *xbar, double *vbar, double *m0bar);
/* Gradients through nsteps integration steps (Limit-sticky9.c:844-893).  pn_adj_forward runs
 * the steps from the current state, keeping the state every checkpoint_every steps on the GPU;
 * the context then holds the final state (read it with pn_get_state to form the loss).
 * pn_adj_backward takes dL/dx(T), dL/dv(T) (host AoS) and returns dL/dx(0), dL/dv(0) and
 * dL/dm0: each segment between checkpoints is recomputed from its checkpoint (stage states and
 * pair sums kept for the segment) and reversed stage by stage, one force VJP per stage.  The
 * context's state is the final state again afterwards. */
int pn_adj_forward(pn_ctx *ctx, int nsteps, int checkpoint_every);
int pn_adj_backward(pn_ctx *ctx, const double *xbar_T, const double *vbar_T, double *xbar_0,
                    double *vbar_0, double *m0bar);

/* ------------------------------------------------------------------ 2b. ensembles */
/* Many independent systems (each a BH + stars, the reference's model) advanced together: one
 * launch per kernel for the whole ensemble, the O(N^2) sweep of every cluster in ONE persistent
 * launch over a shared work queue, each integration step captured in one CUDA graph.  All
 * clusters share dt, inv_c2 and the precision; eps is per cluster.  Arrays are the clusters'
 * AoS arrays concatenated: cluster c occupies rows [sum_{c'<c} n[c'], ... + n[c]), its BH
 * first. */
typedef struct pn_ens pn_ens;
int pn_ens_create(pn_ens **ens, int nclusters, const int *n, const double *eps, const pn_params *p);
int pn_ens_destroy(pn_ens *ens);
int pn_ens_set_state(pn_ens *ens, const double *x, const double *v, const double *m);
int pn_ens_get_state(pn_ens *ens, double *x, double *v);
int pn_ens_force(pn_ens *ens, double *a);
int pn_ens_steps(pn_ens *ens, int nsteps);
int pn_ens_sync(pn_ens *ens);
/* Energies per cluster: out[4c + 0..3] = pot_n, kin_n, pot_pn, total. */
int pn_ens_energy(pn_ens *ens, double *out);
double pn_ens_time(pn_ens *ens);
int pn_ens_last_error(void);
/* Times nsteps captured steps one by one (CUDA events on the ensemble's stream). */
int pn_ens_bench_steps(pn_ens *ens, int nsteps, double *step_ms);
/* Autotuner: per size class (floor(log2 N)) the j-tile size and the j-range of one work item
 * (in tiles), then the launch's i per thread and lanes per i-set, timed on the live state. */
int pn_ens_autotune(pn_ens *ens);
/* Explicit shapes: ipt/js (0 = keep) and, for size_class >= 0, that class's tile size and
 * work-item length. */
int pn_ens_set_shape(pn_ens *ens, int ipt, int js, int size_class, int tile_j, int tiles_per_item);
int pn_ens_get_shape(pn_ens *ens, int size_class, int *ipt, int *js, int *tile_j, int *tiles_per_item);

/* ------------------------------------------------------------------ 3. host utilities */
/* nstars stars uniform in a ball of the given radius (r = R u^(1/3), isotropic), v = 0.
 * x, v: [nstars][3].  Deterministic for a given seed on every platform. */
int pn_ic_uniform_sphere(int nstars, double radius, uint64_t seed, double *x, double *v);
/* nstars stars from a Plummer sphere in Henon units (M = 1, E = -1/4) by the
 * Aarseth-Henon-Wielen (1974) method, shifted to the centre-of-mass frame. */
int pn_ic_plummer(int nstars, uint64_t seed, double *x, double *v);
/* The reference's input format (Limit-sticky9.c:796-809): nstars lines "x y z" then nstars
 * lines "vx vy vz"; values are parsed as float and widened to double, as the reference does.
 * The BH is not in the file. */
int pn_read_init(const char *path, int nstars, double *x, double *v);
int pn_write_init(const char *path, int nstars, const double *x, const double *v);
/* Snapshot block as the reference writes it (Limit-sticky9.c:820-826): n lines of x then n
 * lines of v with "%lf %lf %lf \n".  append != 0 appends to the file. */
int pn_write_snapshot(const char *path, int n, const double *x, const double *v, int append);

/* Number of CUDA devices visible (0 on a machine without a GPU); never aborts. */
int pn_device_count(void);
const char *pn_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PN_H */
