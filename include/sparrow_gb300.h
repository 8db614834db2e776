/*
 * sparrow_gb300.h - C ABI of the GB300 (sm_103a) directional fast-radiosity
 * library (libsparrow_gb300.so).
 *
 * The reference (sparrowpy 1.0.1) is pure Python + numba and has no foreign
 * function interface; each entry point below replaces one of its numba or
 * numpy routines, named in the comment as file:line inside the sparrowpy
 * source tree.  The Python class sparrowpy_gb300.DirectionalRadiosityFast
 * binds these symbols with ctypes (sparrowpy_gb300/_native.py).
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless stated otherwise.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *  - Work is enqueued on `stream`; functions return before it finishes,
 *    except where a comment says the call synchronises.
 *  - Return value: SP_OK (0) or a negative sp_status.  No exception, abort or
 *    device trap crosses the ABI.
 *  - Scratch memory is always caller-provided (`ws`, `ws_bytes`); the
 *    matching *_workspace() function gives the size.  The library itself
 *    calls no cudaMalloc.
 *  - Arrays are C-contiguous, row-major, with the reference's shapes.
 */
#ifndef SPARROW_GB300_H
#define SPARROW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SP_OK = 0,
    SP_ERR_ARG = -1,       /* invalid size, null pointer, unsupported shape */
    SP_ERR_CUDA = -2,      /* a CUDA launch or copy failed */
    SP_ERR_WORKSPACE = -3, /* ws_bytes smaller than the *_workspace() size */
    SP_ERR_RANGE = -4,     /* a delay falls outside the histogram (reference: IndexError) */
    SP_ERR_TIMEOUT = -5,   /* a bounded device wait gave up */
    SP_ERR_UNSUPPORTED = -6
} sp_status;

enum { SP_F32 = 0, SP_F64 = 1 };
enum {
    SP_EXCHANGE_DENSE = 0,
    SP_EXCHANGE_STRUCTURED = 1,
    SP_EXCHANGE_MATERIAL = 2,
    SP_EXCHANGE_SLOTWISE = 3,
    SP_EXCHANGE_GENERAL = 4
};

/* Library version string (static storage). */
const char* sp_version(void);

/* Number of CUDA kernels this library has launched in the process so far
 * (host counter; no GPU work). */
long long sp_kernel_launches(void);

/* ---------------------------------------------------------------- geometry */

/* Patch centres (vertex mean) and areas (fan triangulation).
 * Replaces geometry.py:412-413 `_calculate_center` and :420-448
 * `_calculate_area`.  pts (n, nv, 3) -> centers (n, 3), areas (n). */
int sp_patch_geometry(int n, int nv, const double* pts, double* centers, double* areas, void* stream);

/* Patch-to-patch visibility, upper triangle (i < j) of vis (n, n) as 0/1.
 * Replaces geometry.py:750-797 `_check_patch2patch_visibility` (predicate
 * geometry.py:841-909 `_basic_visibility`); blockers are all n patches. */
size_t sp_patch_visibility_workspace(int n);
int sp_patch_visibility(int n, int nv, const double* centers, const double* normals, const double* pts,
                        uint8_t* vis, void* ws, size_t ws_bytes, void* stream);

/* Allocation-free sp_patch_visibility (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory when visibility is
 * recomputed, e.g. an engine that reserves its whole device budget up front
 * and re-bakes after geometry edits, or a binding without a device allocator
 * of its own, so it has no workspace to pass.  Same arguments and results
 * as sp_patch_visibility, without ws/ws_bytes: the blocker-box scratch is a
 * fixed 405,504-byte array inside this library's device image (reserved
 * when the module loads).  This call allocates nothing.
 *
 * Cost: it runs the single-pass kernel (one pair per thread, the exact FP64
 *   predicate against every blocker box the pair's segment crosses), not
 *   the three-pass form of sp_patch_visibility, whose own-patch pass and
 *   compacted candidate lists need the workspace.  On the 5939-patch street
 *   canyon it takes about 240 ms against about 19 ms.
 * Limit: n <= 16384 patches; larger n returns SP_ERR_WORKSPACE before any
 *   device work (use sp_patch_visibility there).
 * Set-up: the first call on each device, made with that device current,
 *   looks up the array's address (cudaGetSymbolAddress) and keeps it per
 *   device ordinal; make that first call before any stream capture.  A
 *   failed lookup returns SP_ERR_CUDA.  The kept address belongs to the
 *   device's primary context: after cudaDeviceReset, or from a context
 *   made with the driver API, it is stale; use sp_patch_visibility there.
 * Zeroing: nothing has to start at zero (every box read is written earlier
 *   in the same call; vis is cleared on the stream as in sp_patch_visibility).
 * Concurrency: all calls on a device share the one scratch array, so calls
 *   that overlap in time (different streams or host threads) race and give
 *   wrong results; order them on one stream or serialise them. */
int sp_patch_visibility_static(int n, int nv, const double* centers, const double* normals, const double* pts,
                               uint8_t* vis, void* stream);

/* Point-to-patch visibility; blockers are n_surf surfaces (walls).
 * Replaces geometry.py:799-839 `_check_point2patch_visibility`.
 * point (3) -> out (n) 0/1. */
size_t sp_point_visibility_workspace(int n_surf);
int sp_point_visibility(const double* point, int n, const double* centers, int n_surf, int nv,
                        const double* surf_pts, const double* surf_normals, uint8_t* out, void* ws, size_t ws_bytes,
                        void* stream);
/* The same for n_points points (3 each) in one launch: out (n_points, n),
 * row p for points[p] (the receivers of one collection). */
int sp_points_visibility(int n_points, const double* points, int n, const double* centers, int n_surf, int nv,
                         const double* surf_pts, const double* surf_normals, uint8_t* out, void* ws,
                         size_t ws_bytes, void* stream);

/* Row-major list of visible pairs (i < j).  Replaces RadiosityFast.py:377-387.
 * row_counts (n) and row_offset (n+1, int64) are outputs; pairs (n_vis, 2)
 * must hold n*(n-1)/2 entries; pair_index (n, n) (optional) receives the
 * pair number of (i, j) for visible i < j (other entries untouched). */
int sp_visible_pairs(int n, const uint8_t* vis, int32_t* row_counts, int64_t* row_offset, int32_t* pairs,
                     int32_t* pair_index, void* stream);

/* Destination-major list of directed visible pairs (both directions of every
 * visible pair, the loop of RadiosityFast.py:1124-1131).  First call
 * sp_count_directed (sym (n, n) scratch, row_counts (n), row_offset (n+1)),
 * then sp_directed_pairs fills src/dst (row_offset[n] entries, ascending src
 * within each destination). */
int sp_count_directed(int n, const uint8_t* vis, uint8_t* sym, int32_t* row_counts, int64_t* row_offset,
                      void* stream);
int sp_directed_pairs(int n, const uint8_t* sym, const int64_t* row_offset, int32_t* src, int32_t* dst, void* stream);

/* Per directed pair (src -> dst): outgoing-direction index of src toward dst
 * (RadiosityFast.py:402-414 / :1277-1312), incoming index of the BRDF row
 * used by ff_tilde (:1264-1268 / :1359-1390), centre distance (:538-543),
 * normalised-vector length (:1252-1258) and F' (:1255-1256).
 * dirs_in (n_walls, n_in, 3), dirs_out (n_walls, n_out, 3); either may be
 * NULL (index 0 is written). */
int sp_pair_setup(long long n_dir, int n, const int32_t* src, const int32_t* dst, const double* centers,
                  const double* areas, const int32_t* pair_index, const double* ff, const int32_t* wall_of, int n_in,
                  const double* dirs_in, int n_out, const double* dirs_out, int32_t* out_dir, int32_t* in_dir,
                  double* dist, double* unit_len, double* fprime, void* stream);

/* Dense (n, n) int64 outgoing-direction map, `sentinel` where not visible:
 * the reference attribute _patch_2_brdf_outgoing_index (RadiosityFast.py:403-414). */
int sp_outgoing_index_map(long long n_dir, int n, const int32_t* src, const int32_t* dst, const int32_t* out_dir,
                          int64_t sentinel, int64_t* out, void* stream);

/* Dense (n, n) FP64 form-factor matrix from the per-pair values (zero
 * elsewhere): the reference attribute _form_factors (universal.py:42-52). */
int sp_dense_form_factors(long long n_pairs, int n, const int32_t* pairs, const double* ff, double* out, void* stream);

/* Dense ff_tilde (n, n, nd, nb) FP64 from the directed-pair data: replaces
 * RadiosityFast.py:1234-1272 `_form_factors_with_directivity_dim`.  brdf
 * NULL: no BRDF (nd must be 1, factor 1); att NULL: no air attenuation. */
int sp_form_factors_tilde(long long n_dir, int n, int nd, int nb, int n_in, const int32_t* src, const int32_t* dst,
                          const int32_t* in_dir, const double* fprime, const double* unit_len, const double* att,
                          const int32_t* wall_of, const int32_t* brdf_index, const double* brdf, double* out,
                          void* stream);

/* ------------------------------------------------------------ form factors */

/* Universal patch-to-patch form factor for each listed pair (i = source).
 * Replaces universal.py:12-52 `patch2patch_ff_universal` (+ :54-96,
 * integration.py:38-114 Stokes, :116-289 Nusselt).  pts (n_patches, nv, 3):
 * convex planar polygons of nv vertices, 3 <= nv <= 8 (the Nusselt surface
 * samples of a triangle follow integration.py:533-605's triangle branch;
 * polygons of 5 or more vertices are sampled as the parallelogram of their
 * first and last sides, as there).  nv >= 5: FP64 throughout whatever the
 * precision, one warp per pair; method gets 1 or 2 and ws is not used.
 * nv = 3 or 4, precision SP_F64: FP64 throughout.  SP_F32: Stokes re-centred on the patch
 * centres, the second-order terms from FP64 moments and the remainder sum in
 * FP32; FP64 for vertex-sharing pairs (Nusselt), near pairs and pairs whose
 * FP32 error indicator exceeds 5e-6 of the sum.  ff (n_pairs) FP64; method
 * (n_pairs): 0 Stokes FP32, 1 Stokes FP64, 2 Nusselt FP64.  pts holds
 * n_patches patches.  SP_F32 with method needs ws (sp_form_factors_workspace
 * bytes) and synchronises `stream` once; SP_F64, or SP_F32 with method ==
 * NULL, computes FP64 throughout and uses no ws. */
size_t sp_form_factors_workspace(int n_patches, long long n_pairs);
int sp_form_factors(int precision, int n_patches, int nv, long long n_pairs, const int32_t* pairs, const double* pts,
                    const double* normals, const double* areas, double* ff, uint8_t* method, void* ws,
                    size_t ws_bytes, void* stream);

/* Source -> patch energy and directional initial energy.
 * Replaces universal.py:98-147 `_source2patch_energy_universal` and
 * RadiosityFast.py:988-1034 `_add_directional`.  src (3); pts (n, nv, 3),
 * 3 <= nv <= 8; vis (n) from sp_point_visibility; brdf (n_slots, n_in,
 * n_out, nb); outputs e0 (n, nb), d0 (n), e0dir (n, n_out, nb). */
int sp_source_energy(const double* src, int n, const double* centers, const double* pts, int nv, const uint8_t* vis,
                     int nb, const double* att, const int32_t* wall_of, const int32_t* brdf_index, int n_in,
                     const double* dirs_in, int n_out, const double* brdf, double* e0, double* d0, double* e0dir,
                     void* stream);

/* Patch -> receiver factors: point factor (universal.py:149-160), outgoing
 * direction toward the receiver (RadiosityFast.py:728-730) and distance
 * (:712, :745).  rcv (3), pts (n, nv, 3) with 3 <= nv <= 8 -> rfac (n),
 * ridx (n), dist (n). */
int sp_receiver_factors(const double* rcv, int n, const double* centers, const double* pts, int nv,
                        const uint8_t* vis, const int32_t* wall_of, int n_out, const double* dirs_out, double* rfac,
                        int32_t* ridx, double* dist, void* stream);

/* ---------------------------------------------------------- energy exchange */

/* Arguments of sp_energy_exchange (host struct; array members are device
 * pointers).  Directed pairs are destination-major (sp_directed_pairs). */
typedef struct sp_exchange_args {
    int precision;          /* SP_F32 or SP_F64: type of etc_total and of the arithmetic */
    int algorithm;          /* SP_EXCHANGE_DENSE or SP_EXCHANGE_STRUCTURED */
    int n_patches, n_dirs, n_bins, n_samples, max_order;
    const double* energy_0_dir; /* (N, D, B) */
    const double* distance_0;   /* (N) */
    long long n_dir_pairs;
    const int64_t* dst_offset;  /* (N + 1) */
    const int32_t* pair_src;    /* (P) */
    const int32_t* pair_out_dir;/* (P) p2o[src, dst] */
    const int32_t* pair_in_dir; /* (P) BRDF incoming row of the sender */
    const double* pair_distance;/* (P) */
    const double* pair_fprime;  /* (P) F' */
    const double* pair_unit_len;/* (P) */
    const double* air_attenuation; /* (B) or NULL (no attenuation) */
    const int32_t* wall_of;     /* (N) */
    const int32_t* brdf_index;  /* (n_walls) */
    int n_slots, n_in_dirs;
    const double* brdf;         /* (n_slots, n_in, D, B) */
    double speed_of_sound, time_resolution;
    void* etc_total;            /* (N, D, B, T) output, precision type */
    /* structured algorithm only (from sp_brdf_structure): */
    const int32_t* slot_group;  /* (n_slots) material group of each slot */
    const double* slot_scale;   /* (n_slots, B) */
    int n_groups;
    const double* class_diff;   /* (n_groups * n_in, B) */
    const double* class_spec;   /* (n_groups * n_in, B) */
    const int32_t* class_target;/* (n_groups * n_in) mirror direction, -1 if none */
    const int32_t* receiver_order; /* (N) receivers in tile order (16 per tile), NULL = 0..N-1 */
    const int32_t* pair_dst;       /* (P) destination of each directed pair (structured algorithm) */
    int64_t* plan_stats;           /* HOST array of 4 or NULL: source groups, segments, pairs kept, tiles */
    float* order_ms;               /* HOST float or NULL: CUDA-event time of the order loop (all orders) */
    /* structured algorithm, optional (checkpoints for the adjoint; NULL/0 = off): */
    const void* state_in;   /* (N, D, B, T) E_{state_order}: start there instead of at the source energy */
    int state_order;        /* order of state_in (0 without it); orders state_order + 1 .. max_order run */
    void* states_out;       /* (n, N, D, B, T): E_k for k = state_order + i * states_every, i = 0, 1, ...
                               (with state_in, i = 0 is not written: it is state_in) */
    int states_every;
    int skip_total;         /* 1: etc_total is neither cleared nor written */
    /* SP_EXCHANGE_MATERIAL only: per-slot create_from_scattering materials
       BRDF_s[c, o, b] = (1 - alpha[s, b]) (scat[s, b] + (1 - scat[s, b]) gain[c] [o == mirror[c]])
       (brdf, slot_group, slot_scale and class_* are not used; FP32 or FP64) */
    const double* mat_alpha;        /* (n_slots, B) */
    const double* mat_scattering;   /* (n_slots, B) */
    const int32_t* mat_mirror;      /* (n_in) mirror outgoing direction, -1: none */
    const double* mat_gain;         /* (n_in) */
    /* structured / material: nonzero = the caller promises identical pairs and
       materials to every call with the same tag; the plan left in `ws` by the
       previous call with this tag (and these sizes) is then reused */
    long long plan_tag;
    float* scatter_ms;      /* HOST float or NULL: CUDA-event time of the scatter launches alone (all orders) */
    /* structured / material, FP32: E_total's late bins (t >= n_samples / 2, rounded down to a multiple of 4)
       are accumulated over the orders with Kahan compensation; 1 = plain FP32 sums instead */
    int plain_total;
    /* SP_EXCHANGE_GENERAL only: (n_groups * n_in_dirs, D, B) normalised table rows of the classes, with
       BRDF[slot, s, o, b] = slot_scale[slot, b] class_table[slot_group[slot] * n_in + s, o, b] */
    const double* class_table;
    /* SP_EXCHANGE_GENERAL, FP32 with 32 <= D <= 64 and D % 16 == 0: the contraction runs on the tensor cores
       (tcgen05, TF32 with a hi/lo split); 1 = on the CUDA cores instead */
    int no_tensor_cores;
    /* structured / slot-wise / material, FP32: 1 = place E_0 and E_total and build the plan in ws, run no order
       (the orders then run in sp_exchange_batch) */
    int prepare_only;
    /* structured / slot-wise / general / material: 1 = E_total is computed as the last of the partial sums
       S_0 = E_0, S_k = E_0 + M(S_{k-1}) (M: one order's exchange, linear, with the histogram's truncation),
       S_K = E_0 + E_1 + ... + E_K; every order then writes S_k and updates no separate E_total (half the
       order's memory traffic of the mix; no compensation terms).  Needs etc_total and excludes states_out
       and state_in (SP_ERR_ARG); with prepare_only, sp_exchange_batch runs the partial sums.  0 = the
       reference's order: E_k per order, added to E_total */
    int partial_sums;
} sp_exchange_args;

/* Replaces RadiosityFast.py:1073-1145 `_energy_exchange` and :1037-1070
 * `_energy_exchange_init_energy` (max_order < 1).  Synchronises `stream` once
 * (to report SP_ERR_RANGE for a source delay outside the histogram).
 * Algorithms: SP_EXCHANGE_DENSE (any BRDF table, D FMAs per pair and bin);
 * SP_EXCHANGE_STRUCTURED (diffuse-plus-mirror rows, pairs scattered per class
 * (material group, incoming direction), n_classes = n_groups * n_in_dirs <=
 * 256); SP_EXCHANGE_SLOTWISE (the same tables with any number of groups,
 * e.g. per-patch scattering: each pair scattered into a diffuse class and
 * its mirror direction's class, n_classes = 1 + n_dirs; reads the same
 * slot_group / slot_scale / class_* fields); SP_EXCHANGE_GENERAL (any
 * tables, grouped by proportional tables: pairs scattered per class as in
 * the structured algorithm, then each receiver's classes contracted with
 * the full table rows, on the tensor cores for FP32 with n_dirs >= 32;
 * n_classes = n_groups * n_in_dirs <= 256); SP_EXCHANGE_MATERIAL (per-slot
 * absorption and scattering, n_classes = 1 + n_in_dirs). */
size_t sp_energy_exchange_workspace(int precision, int algorithm, int n_patches, int n_dirs, int n_bins,
                                    int n_samples, long long n_dir_pairs, int n_slots, int n_in_dirs,
                                    int n_classes);
int sp_energy_exchange(const sp_exchange_args* args, void* ws, size_t ws_bytes, void* stream);
/* sizeof(sp_exchange_args), for bindings that mirror the struct. */
size_t sp_exchange_args_size(void);

/* ------------------------------------------------------------ energy check */

/* Per-band total energy of E_total (N, D, B, T) in `precision`: out[b] (FP64,
 * device) = sum over patches, directions and bins, accumulated in FP64 in a
 * fixed order (no counterpart in the reference; the FP64 per-band
 * total-energy check).  n_rows = N * D.  ws: sp_energy_totals_workspace(B). */
size_t sp_energy_totals_workspace(int n_bins);
int sp_energy_totals(int precision, long long n_rows, int n_bins, int n_samples, const void* etot, double* out,
                     void* ws, size_t ws_bytes, void* stream);

/* The same totals predicted without time, in FP64: the orders of
 * RadiosityFast.py:1121-1143 summed over t map e_{k-1}[i, o, b] = sum_t
 * E_{k-1} linearly through ff_tilde (:1234-1272), starting from E0dir; the
 * budget is sum_{k <= max_order} sum_{j, o} e_k[j, o, b] -> totals (B, device).
 * It equals sp_energy_totals of the solve's E_total when no contribution is
 * delayed past the histogram (the reference drops those, :1137-1143).  Uses
 * the dense BRDF tables and pair data of `a` (n_dirs * n_bins <= 512);
 * precision, algorithm and the histogram fields are not read.
 * ws: sp_energy_budget_workspace bytes. */
size_t sp_energy_budget_workspace(int n_patches, int n_dirs, int n_bins, long long n_dir_pairs);
int sp_energy_budget(const sp_exchange_args* a, double* totals, void* ws, size_t ws_bytes, void* stream);

/* ------------------------------------------------------------ batched rooms */

/* The exchange orders of many rooms in one persistent launch (no counterpart
 * in the reference, which solves one room per object).  Each room is an
 * sp_exchange_args (FP32, structured / slot-wise / material, at least one
 * pair inside the histogram) already prepared by sp_energy_exchange with
 * prepare_only = 1 in its own workspace; all rooms share n_dirs, n_bins,
 * n_samples (a multiple of 4), max_order and partial_sums.  Blocks take work items (a
 * room's scatter or mix piece of one order) from a device ticket counter and
 * wait, bounded by wait_limit polls (0: 2^24), for the pieces they depend on;
 * a wait that gives up makes the call return SP_ERR_TIMEOUT (the device stays
 * usable).  On success every room's etc_total holds its E_total.
 * window_bins (1024 or 512) and ctas_per_sm (blocks per SM of the persistent
 * grid) are the tile choices an autotuner picks; force_timeout = 1 makes the
 * first item wait for a count that is never reached (a test of the bounded
 * wait).  Synchronises `stream`.  ws: sp_exchange_batch_workspace(n_rooms). */
typedef struct sp_batch_room {
    const sp_exchange_args* args;  /* HOST struct */
    void* ws;                      /* the room's prepared exchange workspace */
    size_t ws_bytes;
} sp_batch_room;

typedef struct sp_batch_args {
    int n_rooms;
    const sp_batch_room* rooms;  /* HOST array */
    int window_bins;
    int ctas_per_sm;
    unsigned wait_limit;
    int force_timeout;
    float* exchange_ms;          /* HOST float or NULL: CUDA-event time of the launch */
    long long* items;            /* HOST or NULL: work items of the launch */
    long long* wait_polls;       /* HOST or NULL: polls the dependency waits of all items took (0: no item waited) */
} sp_batch_args;

size_t sp_exchange_batch_workspace(int n_rooms);
int sp_exchange_batch(const sp_batch_args* args, void* ws, size_t ws_bytes, void* stream);
/* sizeof(sp_batch_args), for bindings that mirror the struct. */
size_t sp_batch_args_size(void);

/* ------------------------------------------------------------------ adjoint */

/* Reverse-mode gradient of the structured exchange, FP32 or FP64 (the
 * precision of the forward arguments `fwd`; no counterpart in
 * the reference, which is not differentiable).  Materials: every slot s uses
 * the create_from_scattering table stored x pi (sparrowpy/brdf.py:8-130,
 * RadiosityFast.py:815): BRDF_s[c, o, b] = (1 - alpha[s, b]) (scattering[s, b]
 * + (1 - scattering[s, b]) mirror_gain[c] [o == mirror_of_in[c]]).  Given
 * dL/d(receiver mono histograms), accumulates dL/dalpha and dL/dscattering
 * of the exchange orders and returns dL/dE0dir for the source term.
 *
 * Use: sp_adjoint_begin once (transposed plan, mu_K = dL/dE_total), then
 * sp_adjoint_order for k = K, K-1, ..., 1 with e_prev = E_{k-1} (in the
 * forward's precision, (N, D, B, T), e.g. from sp_energy_exchange
 * states_out), then
 * sp_adjoint_finish.  The workspace carries the state between the calls;
 * `state` is a HOST struct owned by the caller (zeroed before begin). */
typedef struct sp_adjoint_state {
    int ready;            /* set by sp_adjoint_begin */
    int cur;              /* which internal buffer holds mu_k */
    unsigned n_active;    /* non-empty segments of the transposed plan */
    long long n_groups;   /* source groups of the transposed plan */
} sp_adjoint_state;

typedef struct sp_adjoint_args {
    const sp_exchange_args* fwd;  /* the forward exchange (FP32, structured inputs: pairs, pair_dst,
                                     receiver_order, c, dt, T, distance_0) */
    const int32_t* mirror_of_in;  /* (n_in) mirror outgoing direction of each incoming direction, -1: none */
    const double* mirror_gain;    /* (n_in) K_c */
    const double* alpha;          /* (n_slots, B) */
    const double* scattering;     /* (n_slots, B) */
    int n_receivers;              /* R <= 64 */
    const int32_t* recv_dir;      /* (R, N) outgoing index of each patch toward each receiver */
    const double* recv_factor;    /* (R, N) patch-to-receiver factors (0 where not visible) */
    const double* recv_dist;      /* (R, N) patch-to-receiver distances */
    const double* grad_mono;      /* (R, B, T) dL/d(mono histograms) */
    double* grad_alpha;           /* (n_slots, B), accumulated (+=) */
    double* grad_scattering;      /* (n_slots, B), accumulated (+=) */
    sp_adjoint_state* state;      /* HOST */
} sp_adjoint_args;

size_t sp_adjoint_workspace(int precision, int n_patches, int n_dirs, int n_bins, int n_samples,
                            long long n_dir_pairs, int n_receivers);
int sp_adjoint_begin(const sp_adjoint_args* args, void* ws, size_t ws_bytes, void* stream);
int sp_adjoint_order(const sp_adjoint_args* args, const void* e_prev, void* ws, size_t ws_bytes, void* stream);
int sp_adjoint_finish(const sp_adjoint_args* args, double* grad_e0dir, void* ws, size_t ws_bytes, void* stream);
/* sizeof(sp_adjoint_args), for bindings that mirror the struct. */
size_t sp_adjoint_args_size(void);

/* ------------------------------------------------------ BRDF structure / collection */

/* Structure of the BRDF tables brdf (n_slots, n_in, n_out, nb) for the
 * structured exchange (no counterpart in the reference, which applies the
 * full tables).  Per row (slot, incoming direction): diff (n_slots, n_in, nb)
 * = median over the outgoing directions, target (n_slots, n_in) = the one
 * outgoing direction deviating from diff by more than rel_tol * max|brdf|
 * (-1: none), spec (n_slots, n_in, nb) = that direction's value - diff;
 * scale (n_slots, nb) = max |brdf| per slot and band.  *n_irregular (device
 * int) = rows with more than one deviating direction (the tables are then
 * not of the diffuse-plus-mirror form).  Scratch: ws of
 * sp_brdf_structure_workspace() bytes. */
size_t sp_brdf_structure_workspace(void);
int sp_brdf_structure(int n_slots, int n_in, int n_out, int nb, const double* brdf, double rel_tol, double* diff,
                      double* spec, int32_t* target, double* scale, int* n_irregular, void* ws, size_t ws_bytes,
                      void* stream);

/* One receiver: patchwise (n, nb, nt) and/or mono (nb, nt) FP64 histograms.
 * Replaces RadiosityFast.py:686-752 `_collect_energy_patches` with
 * :1148-1185 `_collect_receiver_energy` (circular roll by ceil(d/c/dt)) and
 * the patch sum of :592.  etot in `precision`. */
size_t sp_collect_workspace(int n_patches, int n_bins);
int sp_collect_receiver(int precision, int n, int nd, int nb, int nt, const void* etot, const int32_t* ridx,
                        const double* rfac, const double* dist, double c, double dt, const double* att,
                        double* patchwise, double* mono, void* ws, size_t ws_bytes, void* stream);

/* ------------------------------------------------------------ Kang solver
 * The legacy Kang radiosity of sparrowpy/classes/RadiosityKang.py in FP64,
 * per wall as the reference runs it.  A wall's histograms are E (nb,
 * n_orders, n, nt) (the reference's E_matrix, n_orders = max order + 1);
 * centres, sizes (Polygon.size) and normals are (.., 3).  `err` (one int,
 * zeroed by the caller) receives 1 when a source delay falls outside the
 * histogram (the reference's IndexError) and 2 when an exchange or receiver
 * delay exceeds it (the ValueError of `_add_delay`). */

/* Replaces RadiosityKang.py:141-207 `init_energy_exchange` with :812-849
 * `_init_energy_exchange`: adds the source energy of each patch at its delay
 * into order 0 of E. */
int sp_kang_init_energy(int n, const double* centers, const double* sizes, const double* normal, const double* src,
                        double sound_power, int nb, const double* absorption, const double* attenuation,
                        double speed_of_sound, double sampling_rate, int n_orders, int nt, double* E, int* err,
                        void* stream);

/* Replaces RadiosityKang.py:269-408 `calculate_form_factor`: ff (n_src,
 * n_rcv) from the source wall's patches to the receiver columns (the other
 * walls' patches in the wall's order); rcv_normals and rcv_wall_centers are
 * per column; max_size is the wall's patch size (used as the patch extent,
 * as the reference does). */
int sp_kang_form_factors(int n_src, const double* src_centers, const double* src_normal, const double* src_wall_center,
                         int n_rcv, const double* rcv_centers, const double* rcv_normals,
                         const double* rcv_wall_centers, double max_size, double* ff, void* stream);

/* Replaces RadiosityKang.py:209-267 `calculate_energy_exchange` for one
 * (receiver wall, source wall) pair at order `order`: adds into E_rcv[:,
 * order] the delayed E_src[:, order - 1] times the source wall's form factors
 * (columns ff_col0 .. ff_col0 + n_rcv of rows of ff_stride) and the receiver
 * wall's scattering, 1 - absorption and exp(-attenuation d).  Calls for the
 * source walls in the receiver wall's order reproduce the reference's sums.
 * ws: sp_kang_exchange_workspace(n_rcv, n_src, nb) bytes. */
size_t sp_kang_exchange_workspace(int n_rcv, int n_src, int nb);
int sp_kang_exchange(int order, int nb, int n_orders, int nt, int n_rcv, const double* rcv_centers, double* E_rcv,
                     const double* scattering, const double* absorption, const double* attenuation, int n_src,
                     const double* src_centers, const double* E_src, const double* ff_src, long long ff_stride,
                     long long ff_col0, double speed_of_sound, double sampling_rate, void* ws, size_t ws_bytes,
                     int* err, void* stream);

/* Replaces RadiosityKang.py:443-498 `energy_at_receiver` of one wall: adds
 * the wall's response (nb, nt) over orders 0 .. max_order into out. */
int sp_kang_receiver(int n, const double* centers, const double* normal, int nb, int n_orders, int nt,
                     const double* E, int max_order, const double* receiver, const double* attenuation,
                     double speed_of_sound, double sampling_rate, double* out, int* err, void* stream);

/* The directional Kang variant (RadiosityKang.py:500-810,
 * PatchesDirectionalKang).  A wall's histograms are E (nb, n_orders, n,
 * n_dirs, nt): one row per patch and outgoing direction of the wall's
 * directional data (the reference's E_matrix is (nb, n_orders, n, nt,
 * n_dirs)).  scat (n_src_dirs, n_dirs, nb) is the receiving wall's
 * directional data (|data| * pi, the reference's directivity_data.freq);
 * scat_idx picks its source-direction row: per patch for the init, per
 * (receiver patch, source patch) pair, row-major, for the exchange.  Both
 * walls of an exchange have the same n_dirs. */

/* Replaces RadiosityKang.py:629-671 `init_energy_exchange`: the plain
 * init's energy at each patch's delay, times |scat[scat_idx[i], d, b]| for
 * every direction d. */
int sp_kang_directional_init_energy(int n, const double* centers, const double* sizes, const double* normal,
                                    const double* src, double sound_power, int nb, const double* absorption,
                                    const double* attenuation, double speed_of_sound, double sampling_rate,
                                    int n_orders, int nt, int n_dirs, const double* scat, const int32_t* scat_idx,
                                    double* E, int* err, void* stream);

/* Replaces RadiosityKang.py:673-745 `calculate_energy_exchange` for one
 * (receiver wall, source wall) pair: as sp_kang_exchange per direction row
 * (scattering is the wall's, all ones in the reference), each term times
 * scat[scat_idx[r * n_src + s], d, b].  ws as sp_kang_exchange. */
int sp_kang_directional_exchange(int order, int nb, int n_orders, int nt, int n_rcv, const double* rcv_centers,
                                 double* E_rcv, const double* scattering, const double* absorption,
                                 const double* attenuation, int n_src, const double* src_centers, const double* E_src,
                                 const double* ff_src, long long ff_stride, long long ff_col0, double speed_of_sound,
                                 double sampling_rate, int n_dirs, const double* scat, const int32_t* scat_idx,
                                 void* ws, size_t ws_bytes, int* err, void* stream);

/* Replaces RadiosityKang.py:747-810 `energy_at_receiver`: as
 * sp_kang_receiver, patch s contributing its row of direction dir_idx[s]
 * (the outgoing direction nearest to the receiver). */
int sp_kang_directional_receiver(int n, const double* centers, const double* normal, int nb, int n_orders, int nt,
                                 const double* E, int max_order, const double* receiver, const double* attenuation,
                                 double speed_of_sound, double sampling_rate, int n_dirs, const int32_t* dir_idx,
                                 double* out, int* err, void* stream);

/* The Kang closed forms of form_factor/kang.py on arbitrary axis-aligned
 * patches (centres, normals (n, 3); sizes (n, size_cols), size_cols 2 or 3,
 * Polygon.size).  Replaces kang.py:12-169 `patch2patch_ff_kang`: ff (n_pairs)
 * of the listed (source, receiver) pairs (pairs (n_pairs, 2)). */
int sp_kang_pair_form_factors(long long n_pairs, const int32_t* pairs, int n, const double* centers,
                              const double* normals, const double* sizes, int size_cols, double* ff, void* stream);

/* Replaces kang.py:171-262 `_source2patch_energy_kang`: energy (n, nb) and
 * distance (n) of each patch from the point source src (3); attenuation
 * (nb) may be NULL (no air attenuation).  sizes (n, 3).  `err` receives 3
 * for a patch whose normal is not along an axis. */
int sp_kang_point_source(int n, const double* src, const double* centers, const double* normals, const double* sizes,
                         int nb, const double* attenuation, double* energy, double* distance, int* err,
                         void* stream);

/* Replaces kang.py:264-277 `_patch2receiver_energy_kang`: factor (n) of each
 * patch for its patch-to-receiver vector (vectors (n, 3)). */
int sp_kang_point_receiver(int n, const double* vectors, const double* normals, double* factor, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPARROW_GB300_H */
