/*
 * gtc.h -- C ABI of the GB300 gravity backend (libgtc.so).
 *
 * This is the drop-in boundary for `device = cuda` behind the reference's
 * gravity/device selection (src/gravity_backends.cpp:139-173). It replaces
 * the Metal context (include/galactic_tides/metal_backend.h:25-54) for the
 * two kernels, and additionally runs the whole grouped solver -- tree build,
 * grouped walk and list evaluation, which the reference does on the host
 * (src/octree.cpp:169-273, src/group_lists.cpp:18-207) -- on the device.
 *
 * Plain C: pointers, sizes and POD structs. Structs that the reference's
 * kernels read have the reference's byte layout (the sizes are the ones
 * static_assert'ed at src/metal/metal_backend.mm:21-24).
 *
 * Errors: every call returns a gtc_status; gtc_last_error() gives the message.
 * The C++ wrapper (galactic-tides_gb300/host/gtc.hpp) turns
 * GTC_INVALID_ARGUMENT into std::invalid_argument and every other failure
 * into std::runtime_error, the exception types the reference uses for the
 * same conditions (gravity_backends.cpp:93-96, metal_backend.mm:206,218-223,
 * 260, group_lists.cpp:25-26,182-183, metal_stub.cpp:15-19).
 *
 * Threading: a context is used from one host thread at a time and owns one
 * CUDA stream and the device buffers it reuses between calls (so calls after
 * the first allocate nothing unless the problem grows), as the reference's
 * Metal context reuses its bindings (metal_backend.mm:58-104).
 */
#ifndef GTC_H
#define GTC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#define GTC_ALIGN16 alignas(16)
#else
#define GTC_ALIGN16 _Alignas(16)
#endif

typedef enum gtc_status {
  GTC_OK = 0,
  GTC_INVALID_ARGUMENT = 1, /* bad sizes or parameters: std::invalid_argument */
  GTC_RUNTIME_ERROR = 2,    /* device failure, 32-bit overflow: std::runtime_error */
  GTC_NO_DEVICE = 3,        /* no usable GB300: std::runtime_error */
  GTC_OUT_OF_MEMORY = 4     /* device allocation failed: std::runtime_error */
} gtc_status;

typedef struct gtc_context gtc_context;

/* kern::float4 (gravity_kernels.h:33-35): 16 bytes, 16-byte aligned. */
typedef struct gtc_float4 {
  GTC_ALIGN16 float x;
  float y, z, w;
} gtc_float4;

/* kern::GTParams (gravity_kernels.h:51-60): 32 bytes, passed by value to
 * the kernels. n = bodies, n_groups = groups (tree kernel), eps2 = softening
 * squared, quadrupole = 1 to include cell quadrupoles. */
typedef struct gtc_kernel_params {
  uint32_t n;
  uint32_t n_groups;
  float G;
  float eps2;
  uint32_t quadrupole;
  uint32_t pad0, pad1, pad2;
} gtc_kernel_params;

/* kern::GTCell (gravity_kernels.h:87-91): centre of mass and mass, then the
 * traceless quadrupole (xx, yy, zz, xy) and (xz, yz, 0, 0). 48 bytes. */
typedef struct gtc_cell {
  gtc_float4 com_mass;
  gtc_float4 q0;
  gtc_float4 q1;
} gtc_cell;

/* kern::GTGroup (gravity_kernels.h:96-105): targets [begin, end) in tree
 * order, cells cell_list[cell_begin, cell_end), bodies
 * body_list[body_begin, body_end). 32 bytes. */
typedef struct gtc_group {
  uint32_t begin, end;
  uint32_t cell_begin, cell_end;
  uint32_t body_begin, body_end;
  uint32_t pad0, pad1;
} gtc_group;

/* Opening criteria for the grouped walk. */
#define GTC_CRITERION_THETA 0   /* the reference's box test (group_lists.cpp:147-154) */
#define GTC_CRITERION_LEARNED 1 /* learned error model, theta test as fallback (below) */

/* GravityParams (octree.h:13-18) plus the make_gravity keys that shape the
 * grouped solver (gravity_backends.cpp:154-160, group_lists.h:64-65). */
typedef struct gtc_gravity_params {
  double G;           /* default 1 */
  double theta;       /* opening angle */
  double eps;         /* Plummer softening length */
  int32_t quadrupole; /* 1: accepted cells carry quadrupoles */
  int32_t group_size; /* 1..32 on the device (GT_SIMD_WIDTH, gravity_backends.cpp:94-96) */
  int32_t leaf_size;  /* bucket size of the octree (default 8) */
  int32_t pack;       /* 1: merge small sibling groups while the run fits a group (the
                         reference's rule, the device default), 0: do not; k >= 2: the
                         packing threshold, runs of at most min(k, group_size) bodies */
  int32_t criterion;  /* GTC_CRITERION_* */
  int32_t reserved;
  double alpha;       /* learned criterion: per-cell error tolerance relative to the
                         group's smallest |a| (ignored by the theta criterion) */
} gtc_gravity_params;

/* GroupTreeGravity::Timings (gravity_backends.h:54-58) and the GroupLists
 * counters (group_lists.h:45-49) of the last call. Times are device times
 * from CUDA events, in milliseconds. */
typedef struct gtc_stats {
  double tree_ms;      /* bounding box, keys, sort, topology, moments, packing */
  double lists_ms;     /* group choice, grouped walk, list offsets */
  double evaluate_ms;  /* list (or direct) evaluation and scatter */
  double total_ms;
  uint64_t cell_interactions; /* summed over targets (group_lists.cpp:197-199) */
  uint64_t body_interactions;
  uint64_t max_list;          /* longest list, cells + bodies */
  uint64_t n_cell_list, n_body_list;
  uint32_t n_nodes, n_groups, max_group, depth;
  double eval_kernel_ms;      /* the list (or direct) evaluation kernel alone */
  uint64_t kernel_launches;   /* kernels this call launched */
  uint64_t walk_tests_fp64;   /* opening tests decided in FP64 (FP32 bound undecided) */
  uint64_t mlp_rows;          /* learned walk: opening tests the network decided */
  uint64_t mlp_batches;       /* learned walk: warp-wide network evaluations */
  uint32_t criterion_used;    /* GTC_CRITERION_* the walk actually used */
  uint32_t graph_steps;       /* leapfrog: steps of the last call replayed from a CUDA graph */
  uint32_t list_passes;       /* walks over the tree for the lists: 1 one pass into per-group
                                 slots, 2 count then fill, learned: the walk's rounds */
  uint32_t spilled_groups;    /* one-pass walk: groups whose lists outgrew their slots and
                                 were written again into the overflow pools */
  uint64_t walk_nodes;        /* node records the walk tested (every round of the learned walk) */
} gtc_stats;

/* Creates a context on CUDA device `device` (GTC_NO_DEVICE if there is
 * none). Replaces metal::Context::Context (metal_backend.mm:122-160). */
gtc_status gtc_create(gtc_context **ctx, int device);
void gtc_destroy(gtc_context *ctx);
/* Message of the last failed call on ctx; with ctx NULL, of the last failed
 * call made without a context (gtc_create, gtc_direct_fp64_noalloc). */
const char *gtc_last_error(const gtc_context *ctx);
const char *gtc_status_name(gtc_status s);
/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order their own work against it. */
void *gtc_stream(gtc_context *ctx);

/* out[i] = (ax, ay, az, potential) of body i against every other, FP32.
 * Host arrays of p->n bodies. Replaces metal::Context::direct
 * (metal_backend.h:39-41, metal_backend.mm:175-207). */
gtc_status gtc_direct(gtc_context *ctx, const gtc_float4 *bodies, const gtc_kernel_params *p,
                      gtc_float4 *out);

/* Evaluates grouped interaction lists: out[i] for every body i in tree
 * order, one group per warp. p->n and p->n_groups must match the arrays and
 * no group may have more than 32 targets (GTC_INVALID_ARGUMENT otherwise).
 * Host arrays. Replaces metal::Context::tree (metal_backend.h:43-49,
 * metal_backend.mm:209-261). */
gtc_status gtc_tree(gtc_context *ctx, const gtc_float4 *bodies, const gtc_cell *cells,
                    uint32_t n_cells, const uint32_t *cell_list, uint64_t n_cell_list,
                    const uint32_t *body_list, uint64_t n_body_list, const gtc_group *groups,
                    const gtc_kernel_params *p, gtc_float4 *out);

/* GroupTreeGravity::compute (gravity_backends.cpp:109-137) entirely on the
 * device: octree with FP64 moments, grouped walk, FP32 list evaluation and
 * scatter back to the caller's order. pos holds n (x, y, z) doubles -- the
 * memory of a std::vector<Vec3> -- and mass n doubles; acc receives n
 * (x, y, z) and pot n. Host pointers; copies are part of the call. */
gtc_status gtc_group_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                           const gtc_gravity_params *gp, double *acc, double *pot);

/* The same with device pointers, enqueued on the context's stream. */
gtc_status gtc_group_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                  uint64_t n, const gtc_gravity_params *gp, double *acc,
                                  double *pot);

/* DirectGravity::compute with the device (gravity_backends.cpp:53-68):
 * bodies packed relative to the bounding-box centre, FP32 tiled kernel,
 * results in the caller's order. Host pointers. */
gtc_status gtc_direct_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                            const gtc_gravity_params *gp, double *acc, double *pot);
gtc_status gtc_direct_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                   uint64_t n, const gtc_gravity_params *gp, double *acc,
                                   double *pot);

/* compute_gravity_tree (src/gravity.cpp:7-26), the `gravity = tree`
 * solver, on the device: the octree, then every body's own walk,
 * Octree::accel_pot (src/octree.cpp:275-344) -- the Barnes (1994) offset
 * criterion with gp->theta, quadrupoles if gp->quadrupole, bodies of opened
 * leaves except the body itself -- in FP64 with the reference's operand
 * order, so the forces are the reference's bit for bit. gp->group_size is
 * not used. gtc_get_stats gives the interactions (cell_interactions,
 * body_interactions = particle interactions). Host pointers (copies are
 * part of the call) or device pointers on the context's stream. */
gtc_status gtc_tree_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                          const gtc_gravity_params *gp, double *acc, double *pot);
gtc_status gtc_tree_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                 uint64_t n, const gtc_gravity_params *gp, double *acc,
                                 double *pot);

/* FP64 direct summation for the m targets idx[0..m) against all n bodies:
 * compute_gravity_direct (src/gravity.cpp:28-45) on a sample, as the
 * reference bench's accuracy judge (apps/galactic_tides_bench.cpp:74-95).
 * Device pointers; acc m x 3, pot m. */
gtc_status gtc_direct_fp64_device(gtc_context *ctx, const double *pos, const double *mass,
                                  uint64_t n, const uint64_t *idx, uint64_t m, double G,
                                  double eps, double *acc, double *pot);

/* The same FP64 sampled sums for callers that cannot allocate device memory:
 * code inside another framework whose caching allocator has reserved the
 * GPU's memory (a cudaMalloc of ours would fail or fragment that pool), and
 * timing-critical loops where cudaMalloc/cudaFree would synchronize the
 * device. No reference counterpart. Needs no context and allocates nothing:
 * the per-slice partial sums live in one fixed 8 MiB device array inside
 * libgtc.so, held by every GPU that loads the library until exit. At most
 * 262144 sample targets (m); larger m is refused (GTC_INVALID_ARGUMENT).
 * idx values must be < n. Enqueued on `stream` (a cudaStream_t, NULL for the
 * legacy default stream) without waiting; the results are ready when the
 * stream reaches that point. The first call in a CUDA context (a device's
 * primary context, normally) looks up the array's address in that context
 * and keeps it under the context's unique id, so a reset device or another
 * context gets a fresh look-up: make that first call before any stream
 * capture. All calls share the array and it keeps the last call's contents
 * (each call writes every slot it reads, nothing needs clearing); calls that
 * overlap on the GPU race on it. A CUDA error already pending from the
 * caller's own work is left in place and the call fails without launching.
 * Errors: gtc_last_error(NULL). */
gtc_status gtc_direct_fp64_noalloc(const double *pos, const double *mass, uint64_t n,
                                   const uint64_t *idx, uint64_t m, double G, double eps,
                                   double *acc, double *pot, void *stream);

gtc_status gtc_get_stats(const gtc_context *ctx, gtc_stats *out);

/* Device times of the last eager gtc_group_force* call's stages, from CUDA
 * events recorded when the context option "stage_events" is 1 (-1 for a
 * stage the call did not time). No reference counterpart: the reference's
 * Timings (gravity_backends.h:54-58) stop at tree / lists / evaluate. */
typedef struct gtc_stage_times {
  double build_ms;     /* tree build start to the walk records (what the walk waits for) */
  double keys_ms;      /* bounding box, split table and keys */
  double sort_ms;      /* the radix sort of the first key word */
  double topology_ms;  /* levels, node count, nodes, children, leaf and tree order */
  double moments_ms;   /* FP64 centres of mass and the walk records (side stream, beside
                          the group choice) */
  double walk_ms;      /* the grouped walk, after the group choice */
  uint32_t sort_passes; /* 8-bit passes of that sort */
  uint32_t reserved;
  double quad_ms;      /* FP64 quadrupoles and the FP32 cells (side stream, beside the walk) */
} gtc_stage_times;
gtc_status gtc_get_stage_times(gtc_context *ctx, gtc_stage_times *out);

/* The accuracy sample of the reference bench (apps/galactic_tides_bench.cpp:
 * 75-79): the indices 0..n-1 in the order std::shuffle leaves them with a
 * std::mt19937_64(seed) engine, the first min(m, n) copied to out. Host only,
 * needs no device. */
void gtc_sample_indices(uint64_t n, uint64_t m, uint64_t seed, uint64_t *out);

/* ---- snapshots (src/snapshot_io.cpp) ------------------------------------
 *
 * The reference writes GADGET-style HDF5 snapshots (write_snapshot /
 * read_snapshot, include/galactic_tides/snapshot_io.h:17-23); HDF5 is not
 * available here, so these keep the same content in a raw binary file
 * (layout in galactic-tides_gb300/host/snapshot.cpp): positions, velocities,
 * masses, IDs, GADGET types (0..5), potentials, the time, the count of each
 * type and free-form "key=value" metadata lines. Host arrays. Particles are
 * written grouped by type in ascending type order (stable within a type), as
 * the reference's reader returns them. id NULL: IDs 0..n-1 in the caller's
 * order; type NULL: all halo (1); pot NULL: zeros. Errors:
 * gtc_last_error(NULL). */
gtc_status gtc_write_snapshot(const char *path, uint64_t n, const double *pos, const double *vel,
                              const double *mass, const uint64_t *id, const uint8_t *type,
                              const double *pot, double time, const char *metadata);
/* The header of a snapshot: particle count, time, count of each type,
 * metadata length in bytes (NULL to skip any). */
gtc_status gtc_snapshot_info(const char *path, uint64_t *n, double *time,
                             uint64_t count_by_type[6], uint64_t *metadata_bytes);
/* Reads a snapshot of n particles (n must match the file; NULL skips an
 * array); metadata receives metadata_bytes bytes, not terminated. */
gtc_status gtc_read_snapshot(const char *path, uint64_t n, double *pos, double *vel, double *mass,
                             uint64_t *id, uint8_t *type, double *pot, char *metadata);

/* ---- time integration (src/integrator.cpp) ----------------------------- */

/* Diagnostics (integrator.h:46-58): potential = 0.5 sum m phi, total =
 * kinetic + potential, virial_ratio = -2 kinetic / potential. */
typedef struct gtc_diagnostics {
  double time, kinetic, potential, total, virial_ratio;
  double momentum[3], angular_momentum[3], centre_of_mass[3];
} gtc_diagnostics;

#define GTC_SOLVER_GROUP 0  /* gtc_group_force_device (theta or learned criterion) */
#define GTC_SOLVER_DIRECT 1 /* gtc_direct_force_device */

/* LeapfrogKDK (integrator.h:31-40, integrator.cpp:5-17) on device arrays:
 * with prime = 1 first computes the forces (prime()), then runs `steps`
 * kick-drift-force-kick steps of dt, FP64 kicks and drifts, on the context's
 * stream; the particles never leave the device. acc and pot hold the forces
 * of the last evaluation. With graph = 1 the whole step (kick, drift,
 * rebuild, evaluation, kick) is replayed as one CUDA graph once the sizes
 * have settled (the group solver with the theta criterion); a step whose
 * tree or lists outgrow the graph's buffers is redone eagerly. gtc_get_stats
 * describes the last force evaluation. */
gtc_status gtc_leapfrog_device(gtc_context *ctx, double *pos, double *vel, const double *mass,
                               double *acc, double *pot, uint64_t n,
                               const gtc_gravity_params *gp, int solver, double dt,
                               uint64_t steps, int prime, int graph);

/* compute_diagnostics (integrator.cpp:19-36) on device arrays, FP64 sums. */
gtc_status gtc_diagnostics_device(gtc_context *ctx, const double *pos, const double *vel,
                                  const double *mass, const double *pot, uint64_t n,
                                  double time, gtc_diagnostics *out);

/* ---- batched ensembles (no reference counterpart) ---------------------- */

/* Independent systems (galaxies) advanced together. When their G, theta,
 * eps, quadrupole flag and leaf size agree (group size and packing may
 * differ), as one forest: every system's bodies in one arena, one tree per
 * system, and each stage of the step (kick and drift, boxes, keys, sort,
 * topology, moments, groups, walk, evaluation, scatter, kick) one launch
 * for all systems; each system moves to the same doubles as on its own.
 * Otherwise (or with option "forest" 0) each system has its own context
 * (stream, workspace), and with graph = 1 one CUDA graph launch replays
 * every system's whole step, the systems' kernel chains running
 * concurrently. */
typedef struct gtc_ensemble gtc_ensemble;
gtc_status gtc_ensemble_create(gtc_ensemble **e, int device, uint32_t systems);
void gtc_ensemble_destroy(gtc_ensemble *e);
/* Message of the last failed call on e (NULL: of gtc_ensemble_create). */
const char *gtc_ensemble_last_error(const gtc_ensemble *e);
/* System i's device arrays (n bodies; acc and pot receive its forces) and
 * grouped-solver parameters (theta criterion). */
gtc_status gtc_ensemble_set_system(gtc_ensemble *e, uint32_t i, double *pos, double *vel,
                                   const double *mass, double *acc, double *pot, uint64_t n,
                                   const gtc_gravity_params *gp);
/* gtc_leapfrog_device for every system: prime, then `steps` steps of dt. */
gtc_status gtc_ensemble_leapfrog(gtc_ensemble *e, double dt, uint64_t steps, int prime,
                                 int graph);
/* System i's context (its stats, exports and options). After a forest
 * leapfrog its stats hold the system's interaction counts, group count and
 * longest list of the last step (no times, no exports). */
gtc_context *gtc_ensemble_context(gtc_ensemble *e, uint32_t i);
/* Ensemble options: "forest" (-1 as one forest when eligible, the default;
 * 1 always, an error when not eligible; 0 never), "walk_warps" (the forest
 * walk: -1 by group count, the default; 0 threads; 1 warps) and
 * "graph_headroom" (the forest's step graph: buffer headroom over the last
 * sizes, default 0.25; a replay that outgrows it, or whose tree needs a
 * second key word, is redone eagerly and the graph captured again). */
gtc_status gtc_ensemble_set_option(gtc_ensemble *e, const char *name, double value);

/* The autotuner: times the grouped solver (theta criterion) on these bodies
 * (device arrays) for group_size 8, 16, 24, 32, each with sibling packing
 * off, packing thresholds group_size / 2 and 3 group_size / 4 and a group's
 * worth (pack 1), each with the walk by threads and by warps, and returns
 * in *best the base parameters with the fastest group_size and pack, in
 * *walk_warps the fastest walk (for option "walk_warps"; NULL to skip) and
 * in *best_ms its mean time per evaluation. The context's own options are
 * left as they were. */
gtc_status gtc_autotune_group(gtc_context *ctx, const double *pos, const double *mass,
                              uint64_t n, const gtc_gravity_params *base,
                              gtc_gravity_params *best, double *best_ms, int *walk_warps);
/* The direct kernel's tile shape: times gtc_direct_force_device on these
 * bodies (device arrays) with 2 and 4 targets per thread, keeps the faster
 * in the context (option "direct_targets") and returns it in *targets, its
 * kernel time in *best_ms. */
gtc_status gtc_autotune_direct(gtc_context *ctx, const double *pos, const double *mass,
                               uint64_t n, const gtc_gravity_params *gp, int *targets,
                               double *best_ms);
/* The list evaluation's tile shape (softened quadrupole evaluation): times
 * the evaluation kernel of gtc_group_force_device on these bodies (device
 * arrays, parameters gp) with 1 and 2 staged pairs per inner iteration and
 * pass costs 8, 16, 24, 32 and 48 (how many slices a group's lists are cut
 * into), keeps the fastest in the context (options "eval_pairs" and
 * "eval_pass_cost") and returns it in *pairs and *pass_cost, its kernel time
 * in *best_ms. The staged pairs do not change the forces; the pass cost
 * changes their summation order only. */
gtc_status gtc_autotune_eval(gtc_context *ctx, const double *pos, const double *mass,
                             uint64_t n, const gtc_gravity_params *gp, int *pairs,
                             int *pass_cost, double *best_ms);

/* ---- tuning and diagnostics (no reference counterpart) ------------------ */

/* Sets an option of the context:
 *   "walk_split_depth"   0, 1 or 2 (default 0): each group's walk runs as
 *                        independent tasks, one per subtree at this depth
 *                        (0: one task per group; measured fastest on GB300).
 *                        Results do not depend on it.
 *   "learned_guard_theta" > 0 (default 1.5): the learned walk opens every
 *                        cell closer than 2 h / guard + delta (the theta
 *                        test with this angle guards the network).
 *   "learned_band"       >= 0 log2 units, or < 0 for the model's own band
 *                        (default): tests whose centred error prior lies
 *                        further than this from the tolerance are decided by
 *                        it; the rest go to the network (0: prior only).
 *   "learned_walk_budget" whole number >= 0 (default 576): in the learned
 *                        walk's first round a thread tests this many nodes
 *                        for its group, then a warp walks the rest 32 nodes
 *                        at a time (0: the thread walks it all). The lists
 *                        hold the same entries; only their order depends on it.
 *   "learned_pair_budget" the same for the later rounds (default 48), which
 *                        walk the subtrees of the pairs the network opened.
 *   "learned_read_every_round" 0 (default) or 1: the learned walk first runs
 *                        as many rounds as its last call needed, then reads
 *                        back how many pairs the last one deferred (more
 *                        rounds follow one read back each); 1 reads back
 *                        after every round. Results do not depend on it.
 *   "walk_warps"         -1 (default), 0 or 1: the plain walk by warps, one
 *                        per group, 32 node tests per step (1), or by
 *                        threads, two per group in the one-pass walk (0),
 *                        whose lists keep the reference's order; -1 takes
 *                        warps below 40000 groups (the thread walk leaves
 *                        the GPU idle there) and threads above (neighbouring
 *                        groups share their record loads). Lists hold the
 *                        same entries.
 *   "learned_warps"      -1 (default), 0 or 1: the learned walk's rounds by
 *                        warps, one per group (1), or by three threads per
 *                        group with the long walks handed to warps (0, the
 *                        budgets below); -1 picks as "walk_warps" does.
 *   "eval_pairs"         2 (default) or 1: staged pairs each lane of the list
 *                        evaluation works per inner iteration (the forces do
 *                        not depend on it; gtc_autotune_eval picks it).
 *   "eval_pass_cost"     whole number 1..256 (default 24): a pass's fixed cost
 *                        in staged entries per lane, from which the list
 *                        evaluation picks how many slices to cut each group's
 *                        lists into (summation order only; gtc_autotune_eval
 *                        picks it).
 *   "direct_targets"     2 (default) or 4: targets per thread of the direct
 *                        kernel (its tile shape; gtc_autotune_direct picks it).
 *   "stage_events"       0 (default) or 1: record CUDA events at the stage
 *                        boundaries of eager group solves (gtc_get_stage_times).
 *   "graph_headroom"     0..4 (default 0.25): a leapfrog graph is captured
 *                        with buffers this fraction larger than the last
 *                        solve's tree and lists (0: exactly those sizes, so
 *                        most changes abort the replay and redo it eagerly).
 * GTC_INVALID_ARGUMENT for an unknown name or a value out of range. */
gtc_status gtc_set_option(gtc_context *ctx, const char *name, double value);

/* Measured FP32 FMA throughput of this GPU in TFLOP/s (one FMA = 2 flops):
 * the roofline denominator for the FP32 evaluation kernels. */
gtc_status gtc_measure_fp32_peak(gtc_context *ctx, double *tflops);

/* ---- learned opening criterion (no reference counterpart) ---------------
 *
 * Replaces the accept test of the grouped walk (group_lists.cpp:147-154)
 * when gtc_gravity_params.criterion is GTC_CRITERION_LEARNED. A 6-64-64-1
 * ReLU network corrects a physical prior for the force error that accepting
 * a cell would cause for a group (log2 of the largest |a_multipole - a_exact|
 * over the group's targets, in units of G M_total / L^2, L the root
 * half-size):
 *   prediction = prior + y_mean + y_std * net((f - mean) / std)
 *   prior      = log2(2 * 3^1.5) + f3 + 3 f1 - 5 f2
 * with features f0 log2(group half-extent / L), f1 log2(cell half-size / L),
 * f2 log2(distance from the group box to the cell's centre of mass / L),
 * f3 log2(cell mass / M_total), f4 log2(|Q| / (M L^2)), f5 delta / half.
 * A cell is accepted when the prediction is below
 * log2(alpha * a_g * L^2 / (G M_total)), a_g = max(min |a|, mean |a| / 2)
 * over the group's targets, |a| from the context's previous solve of the
 * same bodies (caller order). Cells inside the guard (learned_guard_theta) are always opened.
 * The walk defers the pairs the prior cannot settle; the network decides
 * them in dense batches in BF16 on the tensor cores (mma.sync), FP32
 * accumulation, and the walk continues under the cells it opens.
 * Fallback: with no model, or no previous solve of the same n, the call runs
 * the theta walk (gtc_stats.criterion_used says which ran). Every solve of a
 * context with a model records |a| for the next.
 *
 * Model layout (GTC_LEARNED_MODEL_FLOATS floats): W1[6][64], b1[64],
 * W2[64][64], b2[64], W3[64], b3 (W[in][out]), then mean[6], std[6], y_mean,
 * y_std, band (log2 units; tests whose centred prior, prior + y_mean, lies
 * further than band from the tolerance are decided by it alone). */
#define GTC_LEARNED_FEATURES 6
#define GTC_LEARNED_PARAMS 4673
#define GTC_LEARNED_MODEL_FLOATS 4688

/* Training samples from the bodies (host arrays): builds the tree and groups
 * with gp, walks sampled groups with opening angle theta_gen and labels every
 * visited cell of more than two bodies beyond the guard angle theta_guard
 * by FP64 direct summation over its bodies (cells of more than
 * max_cell_bodies bodies are skipped). Appends at most max_new samples;
 * *added receives the count. */
gtc_status gtc_learned_add_samples(gtc_context *ctx, const double *pos, const double *mass,
                                   uint64_t n, const gtc_gravity_params *gp, double theta_gen,
                                   double theta_guard, uint64_t max_new,
                                   uint32_t max_cell_bodies, uint64_t *added);
gtc_status gtc_learned_sample_count(const gtc_context *ctx, uint64_t *count);
/* Copies samples [first, first + count) (NULL to skip an array): feat
 * count x 6, label count, pairs count x 2 = (group, node) in the tree and
 * groups of the call that made the sample (gtc_group_export numbering when
 * the same bodies and parameters are solved with the theta criterion). */
gtc_status gtc_learned_export_samples(gtc_context *ctx, uint64_t first, uint64_t count,
                                      float *feat, float *label, uint32_t *pairs);
gtc_status gtc_learned_clear_samples(gtc_context *ctx);

/* Trains the context's model on its samples with the project's own kernels:
 * `steps` Adam steps (learning rate lr) on random minibatches of `batch`
 * samples, mean squared error of the correction in normalised units. With
 * init = 1 first sets the normalisation from the samples and draws new
 * weights from `seed`. Afterwards sets the band to the 0.99 quantile of
 * |y_std net| over the samples. *loss: the last minibatch's loss. */
gtc_status gtc_learned_train(gtc_context *ctx, uint64_t steps, uint32_t batch, float lr,
                             uint64_t seed, int init, double *loss);
/* Gradient of the mean squared error of the given model (host,
 * GTC_LEARNED_MODEL_FLOATS) on n given samples (host), by the training
 * kernels: grad (GTC_LEARNED_PARAMS floats) and *loss. The context's own
 * model is left as it was. */
gtc_status gtc_learned_gradient(gtc_context *ctx, const float *model, const float *feat,
                                const float *label, uint32_t n, float *grad, double *loss);
gtc_status gtc_learned_set_model(gtc_context *ctx, const float *model);
gtc_status gtc_learned_get_model(gtc_context *ctx, float *model);
/* The walk's BF16 tensor-core inference on n given feature rows (host):
 * pred[i] = predicted log2 error. */
gtc_status gtc_learned_predict(gtc_context *ctx, const float *feat, uint64_t n, float *pred);

/* ---- exports of the last gtc_group_force*, for parity checks ------------ */

/* One node of the device octree. Nodes are numbered in the order the
 * reference's walk visits them (depth first, children last octant first), so
 * node `skip` is the first node after this node's subtree. The fields of
 * Octree::Node (octree.h:52-63) are all here; children are the nodes
 * i+1, skip[i+1], ... up to skip[i] (last octant first). */
typedef struct gtc_node {
  double center[3];
  double half;
  double com[3];
  double mass;
  double quad[6];
  double delta;
  uint32_t begin, end;
  uint32_t skip;
  uint32_t parent;
  int32_t depth;
  int32_t n_children;
} gtc_node;

/* Sizes of the last group call's tree and lists (for sizing the export). */
gtc_status gtc_group_sizes(const gtc_context *ctx, uint64_t *n_bodies, uint64_t *n_nodes,
                           uint64_t *n_groups, uint64_t *n_cell_list, uint64_t *n_body_list);
/* Copies the tree (NULL to skip any array): nodes, order (tree position ->
 * caller index), the FP32 bodies and cells the evaluator read, the groups
 * and both lists, the tree-order evaluator output. The lists are laid out
 * as the reference's GroupLists (group_lists.h:37-55): groups back to back,
 * each group's cells in the reference's order. Each group's bodies are the
 * reference's; the walk by warps (the default, option walk_warps) writes
 * them in the order its steps reach them and the export gives them in
 * ascending order, the walk by threads in the reference's order. */
gtc_status gtc_group_export(gtc_context *ctx, gtc_node *nodes, uint64_t *order,
                            gtc_float4 *bodies, gtc_cell *cells, gtc_group *groups,
                            uint32_t *cell_list, uint32_t *body_list, gtc_float4 *out);

#ifdef __cplusplus
}
#endif

#endif /* GTC_H */
