/*
 * splinegrids_b200.h -- C ABI of libsplinegrids_b200.so, the GB300 (sm_103a) grid
 * evaluation hot path of SplineGrids.jl.
 *
 * Every entry point replaces one KernelAbstractions launch (or one public function)
 * of the reference, SouthEndMusic/SplineGrids.jl v0.1.1; the citation above each
 * declaration names it.  Julia host code binds these with `ccall`; the Python package
 * in splinegrids.jl_gb300/splinegrids binds them with ctypes.
 *
 * Conventions (all taken from the reference's data layout):
 *   - arrays are device pointers in Julia column-major order, first index fastest;
 *     the output dimension Nout is the slowest index of control points and eval;
 *   - sample indices are 1-based int32 (`Ti = Int32`, the reference default);
 *   - a basis table is the reference's `eval[n_samples, degree+1, max_deriv+1]`;
 *   - a RefinementMatrix is the reference's 1-based banded format (row_pointer,
 *     column_start, nzval);
 *   - dimension numbers passed as arguments (dims_refinement) are 0-based;
 *   - every call is asynchronous on the given stream (NULL = the legacy default
 *     stream) unless its comment says it synchronizes; nothing on the evaluate /
 *     adjoint / refinement paths allocates memory.  Plans allocate at creation.
 *   - return value: SG_OK or an SG_ERR_* code; sg_last_error() gives the message
 *     of the calling thread's last failure.
 */
#ifndef SPLINEGRIDS_B200_H
#define SPLINEGRIDS_B200_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *sg_stream_t; /* == cudaStream_t */

/* Status codes. */
#define SG_OK 0
#define SG_ERR_INVALID_ARGUMENT 1 /* bad shape, pointer, degree, derivative order */
#define SG_ERR_UNSUPPORTED 2      /* e.g. adjoint of a NURBS grid (src/adjoint.jl:57) */
#define SG_ERR_CUDA 3             /* a CUDA runtime call failed */
#define SG_ERR_TIMEOUT 4          /* a bounded device wait gave up */
#define SG_ERR_OUT_OF_MEMORY 5    /* plan creation could not allocate */
#define SG_ERR_DEVICE_CHECK 6     /* a device-side check recorded bad input */

/* Value types (`Tv` of the reference). */
#define SG_F64 0       /* Float64 everything */
#define SG_F32 1       /* Float32 everything (the reference default) */
#define SG_BF16_F32 2  /* control points stored bfloat16; basis, eval, accumulation Float32 */

#define SG_MAX_NIN 8      /* input dimensions supported */
#define SG_MAX_DEGREE 15  /* spline degree supported */

int sg_version(void);
const char *sg_last_error(void);

/* ------------------------------------------------------------------ SplineDimension */

/* KnotVector(knot_values, multiplicities): expand_knot_vector_kernel,
 * src/knot_vector.jl:21-49 and src/util_kernels.jl:1-20.
 * knots_all has n_knots = sum(multiplicities) entries (the caller allocates it, as
 * the reference's `similar(knot_values, sum(multiplicities))`). dtype SG_F32/SG_F64. */
int sg_expand_knots(int32_t dtype, const void *knot_values, const int32_t *multiplicities,
                    int64_t n_values, int64_t n_knots, void *knots_all, sg_stream_t stream);

/* set_sample_indices!: src/utils.jl:19-29 and set_sample_indices_kernel,
 * src/util_kernels.jl:22-49.  sample_indices[l] = clamp(#{knots_all <= t_l},
 * degree+1, n_knots-degree-1), 1-based, bit-exact with the reference's linear scan. */
int sg_sample_indices(int32_t dtype, const void *sample_points, int64_t n_samples,
                      const void *knots_all, int64_t n_knots, int32_t degree,
                      int32_t *sample_indices, sg_stream_t stream);

/* evaluate!(::SplineDimension): src/spline_dimension.jl:231-243 and
 * spline_dimension_kernel, src/spline_dimension.jl:160-215 (Cox-de Boor values and
 * derivatives).  eval is [n_samples, degree+1, max_derivative_order+1]; computed in
 * Float64 and stored as dtype. */
int sg_basis_eval(int32_t dtype, const void *knots_all, int64_t n_knots,
                  const void *sample_points, const int32_t *sample_indices, int64_t n_samples,
                  int32_t degree, int32_t max_derivative_order, void *eval,
                  sg_stream_t stream);

/* decompress(::SplineDimension; derivative_order): src/spline_dimension.jl:251-272 and
 * decompress_basis_function_eval_kernel, src/util_kernels.jl:51-67.  out is the dense
 * [n_samples, n_basis] matrix; entries outside the support are written as zero. */
int sg_decompress(int32_t dtype, const void *eval, const int32_t *sample_indices,
                  int64_t n_samples, int32_t degree, int32_t max_derivative_order,
                  int32_t derivative_order, int64_t n_basis, void *out, sg_stream_t stream);

/* ------------------------------------------------------------------ SplineGrid */

/* What a SplineGrid / NURBSGrid hands to its kernels (src/spline_grid.jl:19-117,
 * :211-214): per input dimension the sample indices and the basis table. */
typedef struct sg_grid_desc {
    int32_t nin;          /* input dimensions, 1..SG_MAX_NIN */
    int32_t nout;         /* output channels (Nout; fold control-point sets in here) */
    int32_t dtype;        /* SG_F64 / SG_F32 / SG_BF16_F32 */
    int32_t has_weights;  /* 1 for a NURBSGrid */
    int64_t n_samples[SG_MAX_NIN];
    int64_t n_basis[SG_MAX_NIN];           /* control points per dim */
    int32_t degree[SG_MAX_NIN];
    int32_t max_derivative_order[SG_MAX_NIN];
    const int32_t *sample_indices[SG_MAX_NIN];  /* device, 1-based */
    const void *basis_eval[SG_MAX_NIN];         /* device, [ns, d+1, maxd+1] */
} sg_grid_desc;

typedef struct sg_grid_plan sg_grid_plan;

/* Build a plan for one grid: validates the descriptor, reads the sample indices once
 * (synchronizes `stream`) to check their range and order, and allocates the
 * intermediate buffers of the separable passes.  The reference has no plan object;
 * its SplineGrid constructor (src/spline_grid.jl:34-57) is where a Julia wrapper
 * creates one. */
int sg_grid_plan_create(const sg_grid_desc *desc, sg_stream_t stream, sg_grid_plan **plan);

/* Re-read the sample indices after they changed (set_sample_indices!); synchronizes. */
int sg_grid_plan_refresh(sg_grid_plan *plan, sg_stream_t stream);

void sg_grid_plan_destroy(sg_grid_plan *plan);

/* Bytes of device scratch the plan holds. */
int64_t sg_grid_plan_workspace_bytes(const sg_grid_plan *plan);

/* Per-pass CUDA-event timing (no counterpart in the reference, which has no
 * profiling; it serves the roofline measurement).  When enabled, every evaluate /
 * evaluate_adjoint call records an event pair around each of its kernel launches on
 * the call's stream.  sg_grid_plan_pass_times synchronizes on the last call's events
 * and writes the duration in ms of each pass, in launch order, to ms[0..*n_passes-1]
 * (*n_passes in: capacity, out: number of passes of the last call). */
int sg_grid_plan_enable_timing(sg_grid_plan *plan, int32_t enable);
int sg_grid_plan_pass_times(sg_grid_plan *plan, float *ms, int32_t *n_passes);

/* Status of the plan's earlier launches on `stream` (no counterpart in the reference,
 * whose kernels have no device-side waits).  The adjoint passes over axes k >= 1 wait
 * on shared-memory barriers for their bulk copies; each wait gives up after a bounded
 * time and records SG_ERR_TIMEOUT in the plan's status word instead of hanging.
 * Synchronizes `stream`, returns that status and clears it. */
int sg_grid_plan_check(sg_grid_plan *plan, sg_stream_t stream);

/* Measured tuning of the adjoint: for every pass over an axis k >= 1 the plan times
 * candidate chunk sizes of the bulk-copy stream (8..64 control points per tile, three
 * runs each, on `stream`, with the caller's cotangent eval_bar and gradient buffer
 * control_points_bar as scratch) and keeps the fastest for later sg_evaluate_adjoint
 * calls; chosen[k] (optional, SG_MAX_NIN entries) receives the choice (0: the built-in
 * heuristic, e.g. for axis 0).  Results are bitwise the same for every choice.
 * Synchronizes `stream`.  sg_grid_plan_untune returns to the heuristic. */
int sg_grid_plan_tune(sg_grid_plan *plan, const int32_t *derivative_order, const void *eval_bar,
                      void *control_points_bar, sg_stream_t stream, int32_t *chosen);
int sg_grid_plan_untune(sg_grid_plan *plan);

/* Evaluation strategy of a plan (no counterpart in the reference, whose evaluate! and
 * evaluate_adjoint! launch one kernel per call: src/spline_grid.jl:216-228,
 * src/adjoint.jl:70-81).  SG_STRATEGY_SEPARABLE contracts one axis per launch through
 * the plan's scratch; SG_STRATEGY_FUSED (grids with Nin = 2, degrees <= 3, no weights,
 * fewer than 2^31 values) contracts both axes in one launch with nothing intermediate
 * in device memory (its adjoint also needs sorted samples on both axes).  Both give
 * bitwise identical results.  SG_STRATEGY_AUTO (the default) takes the fused path
 * wherever it applies.  sg_grid_plan_set_strategy(FUSED) on a grid outside it returns
 * SG_ERR_UNSUPPORTED; sg_grid_plan_paths reports the path each direction takes.  On
 * the fused path sg_grid_plan_tune times adjoint tile sizes instead of stream chunks
 * (chosen[1] = axis-1 control points per tile). */
#define SG_STRATEGY_AUTO 0
#define SG_STRATEGY_SEPARABLE 1
#define SG_STRATEGY_FUSED 2
int sg_grid_plan_set_strategy(sg_grid_plan *plan, int32_t strategy);
int sg_grid_plan_paths(const sg_grid_plan *plan, int32_t *forward, int32_t *adjoint);

/* evaluate!(spline_grid; derivative_order, control_points, eval):
 * src/spline_grid.jl:200-230 and spline_eval_kernel, src/spline_grid.jl:119-183.
 * control_points [n_basis..., nout] (bfloat16 for SG_BF16_F32), weights [n_basis...]
 * or NULL (required iff has_weights), eval [n_samples..., nout].
 * derivative_order: host array of nin ints; NURBS grids accept only zeros
 * (src/validation.jl:67-74). */
int sg_evaluate(sg_grid_plan *plan, const int32_t *derivative_order,
                const void *control_points, const void *weights, void *eval,
                sg_stream_t stream);

/* evaluate! for several derivative orders of the same control points in one call:
 * eval_i = evaluate!(grid; derivative_order = orders[i*nin .. i*nin+nin-1]).  No single
 * reference call does this; its optics and PDE examples call evaluate! once per order
 * (docs/src/examples_optics.md:189-191, docs/src/examples_pde.md:69-72).  Each distinct
 * prefix (orders along axes 0..k) is contracted once and shared by the orders below it,
 * so e.g. (0,0), (1,0), (0,1) run 5 passes instead of 6 and read the control points
 * twice instead of three times.  Results are bitwise those of separate sg_evaluate calls.
 * Nin = 1 and Nin > 3 run one sg_evaluate per order.  Errors as sg_evaluate, per order. */
int sg_evaluate_multi(sg_grid_plan *plan, int32_t n_orders, const int32_t *orders,
                      const void *control_points, const void *weights, void *const *evals,
                      sg_stream_t stream);

/* evaluate_adjoint!(spline_grid; derivative_order, control_points, eval):
 * src/adjoint.jl:52-83 and spline_eval_adjoint_kernel, src/adjoint.jl:1-40.
 * Overwrites control_points_bar [n_basis..., nout] with M' * eval_bar.  Gather form:
 * each control point sums its sample support in a fixed order, without atomics, so
 * the result is bitwise deterministic.  NURBS: SG_ERR_UNSUPPORTED, as the reference.
 * For SG_BF16_F32 grids eval_bar and control_points_bar are Float32. */
int sg_evaluate_adjoint(sg_grid_plan *plan, const int32_t *derivative_order,
                        const void *eval_bar, void *control_points_bar, sg_stream_t stream);

/* ------------------------------------------------------------------ refinement */

/* RefinementMatrix, src/refinement_matrix.jl:19-57 (device arrays, 1-based). */
typedef struct sg_refmat {
    int64_t m;                    /* rows */
    int64_t n;                    /* columns */
    int64_t nnz;                  /* length(nzval) */
    const int32_t *row_pointer;   /* [m] */
    const int32_t *column_start;  /* [m] */
    const void *nzval;            /* [nnz], dtype */
} sg_refmat;

/* mult!(Y, As, B, dims_refinement): src/refinement_matrix.jl:421-445 and
 * refinement_matrix_array_mul_kernel, src/refinement_matrix.jl:365-403.
 * Y[I] = sum_J B[J] prod_r As[r][I_dims[r], J_dims[r]]; size_Y/size_B have ndims
 * entries (control-point dims and Nout); dims_refinement 0-based. */
int sg_mult(int32_t dtype, int32_t ndims, const int64_t *size_Y, const int64_t *size_B,
            int32_t n_refmat, const sg_refmat *As, const int32_t *dims_refinement,
            const void *B, void *Y, sg_stream_t stream);

/* mult_adjoint!(B, As, Y, dims_refinement): src/adjoint.jl:127-152 and
 * refinement_matrix_array_mul_adjoint_kernel, src/adjoint.jl:85-125.  Overwrites B.
 * Gather form (each B entry sums the rows that cover it), deterministic. */
int sg_mult_adjoint(int32_t dtype, int32_t ndims, const int64_t *size_Y,
                    const int64_t *size_B, int32_t n_refmat, const sg_refmat *As,
                    const int32_t *dims_refinement, const void *Y, void *B,
                    sg_stream_t stream);

/* local_refinement_kernel, src/control_points.jl:296-311:
 * control_points[refinement_indices[i, :]..., o] = refinement_values[i, o].
 * refinement_indices [n_refined, nin] 1-based int32, refinement_values [n_refined, nout].
 * Indices must be unique (activate_local_refinement! makes them so). */
int sg_local_refinement(int32_t dtype, int32_t nin, int32_t nout, const int64_t *cp_size,
                        int64_t n_refined, const int32_t *refinement_indices,
                        const void *refinement_values, void *control_points,
                        sg_stream_t stream);

/* local_refinement_adjoint_kernel, src/adjoint.jl:154-170: gather
 * refinement_values[i, o] = control_points[idx_i..., o], then zero those entries. */
int sg_local_refinement_adjoint(int32_t dtype, int32_t nin, int32_t nout,
                                const int64_t *cp_size, int64_t n_refined,
                                const int32_t *refinement_indices, void *refinement_values,
                                void *control_points, sg_stream_t stream);

/* ------------------------------------------------------------------ batched grids */

/* Many grids of uneven sizes (each with its own control-point sets folded into nout)
 * evaluated forward and/or adjoint in ONE persistent launch fed by a device-side work
 * queue.  No counterpart in the reference, which evaluates one grid per call
 * (evaluate!, src/spline_grid.jl:200-230; evaluate_adjoint!, src/adjoint.jl:52-83);
 * per grid the results are those of sg_evaluate / sg_evaluate_adjoint.
 * Non-NURBS grids of degree <= 3, all SG_F32 or all SG_F64.
 * derivative_orders: host array [n_grids][SG_MAX_NIN].  Creation reads every grid's
 * sample indices (synchronizes) and allocates the per-grid intermediates. */
typedef struct sg_batch_plan sg_batch_plan;

int sg_batch_plan_create(int32_t n_grids, const sg_grid_desc *grids,
                         const int32_t *derivative_orders, sg_stream_t stream,
                         sg_batch_plan **plan);

/* Host arrays of n_grids device pointers: control points and eval (forward), eval_bar
 * and control_points_bar (adjoint); either pair may be NULL.  Builds and uploads the
 * work queue (synchronous); call again when the arrays move. */
int sg_batch_set_arrays(sg_batch_plan *plan, const void *const *control_points,
                        void *const *evals, const void *const *eval_bars,
                        void *const *control_points_bars);

#define SG_BATCH_FORWARD 1
#define SG_BATCH_ADJOINT 2

/* One launch over every grid: what = SG_BATCH_FORWARD, SG_BATCH_ADJOINT or both
 * (OR-ed).  Asynchronous and capturable in a CUDA graph (two memsets + one kernel). */
int sg_batch_run(sg_batch_plan *plan, int32_t what, sg_stream_t stream);

/* Synchronizes `stream` and returns SG_ERR_TIMEOUT if a bounded device-side dependency
 * wait of the last run gave up (its tiles were skipped), else SG_OK. */
int sg_batch_check(sg_batch_plan *plan, sg_stream_t stream);

/* Strategy of the batch (SG_STRATEGY_*, see sg_grid_plan_set_strategy).  With AUTO (the
 * default) every grid with Nin = 2, degrees <= 3, sorted samples and fewer than 2^31
 * values runs fused: its forward as independent warp tasks (one launch for all such
 * grids), its adjoint as tiles that contract both axes (one persistent launch fed by a
 * device work queue), with no intermediates in device memory.  The other grids run the
 * separable passes from the dependency-ordered queue, in a further launch.  SEPARABLE
 * puts every grid in that queue (allocating the intermediates the fused grids skip).
 * Results are bitwise the same either way.  Rebuilds the work lists when arrays are set
 * (synchronous).  sg_batch_fused_grids counts the grids on the fused path.  No
 * counterpart in the reference (one grid per evaluate! call). */
int sg_batch_set_strategy(sg_batch_plan *plan, int32_t strategy);
int64_t sg_batch_fused_grids(const sg_batch_plan *plan);

/* Measured tuning of the fused units' sizes (no counterpart in the reference): the
 * forward (eval values per warp task) and the adjoint (cotangent values per tile, 0 =
 * axis 1 whole) are each timed over candidate sizes, three runs each on `stream` with
 * the plan's arrays (which it overwrites: eval and gradients), and the fastest is kept
 * for later runs; chosen (optional, 2 entries) receives the two sizes.  Results are
 * bitwise the same for every size.  Synchronizes `stream`.  sg_batch_set_unit_sizes
 * sets them explicitly (<= 0: the built-in size). */
int sg_batch_tune(sg_batch_plan *plan, sg_stream_t stream, int64_t *chosen);
int sg_batch_set_unit_sizes(sg_batch_plan *plan, int64_t forward_values, int64_t adjoint_values);

/* Per-kind cycle profile of the persistent kernel (no counterpart in the reference;
 * it serves the roofline measurement).  While enabled, every queue item adds to
 * device counters, per pass kind k (0 forward axis 0, 1 forward axis >= 1, 2 adjoint
 * axis >= 1 by warp tasks, 3 adjoint axis 0, 4 adjoint axis >= 1 by bulk-copy
 * stream): out[3k] = SM cycles from taking the item until its dependency was met,
 * out[3k+1] = SM cycles of the item's work, out[3k+2] = items.  sg_batch_profile
 * synchronizes `stream`, copies the SG_BATCH_PROFILE_WORDS counters to out and
 * clears them. */
#define SG_BATCH_PROFILE_WORDS 15
int sg_batch_enable_profile(sg_batch_plan *plan, int32_t enable);
int sg_batch_profile(sg_batch_plan *plan, sg_stream_t stream, int64_t *out);

void sg_batch_plan_destroy(sg_batch_plan *plan);
int64_t sg_batch_plan_workspace_bytes(const sg_batch_plan *plan);
int64_t sg_batch_items(const sg_batch_plan *plan, int32_t what);  /* queue length */

/* n asynchronous copies dst[i] <- src[i] of bytes[i] bytes on `stream`, one
 * cudaMemcpyAsync each (host/device resolved by unified addressing; pinned host memory
 * for asynchrony): the uploads or downloads of a host-data batch step in one call. */
int sg_copy_list(int64_t n, void *const *dst, const void *const *src, const int64_t *bytes,
                 sg_stream_t stream);

/* ------------------------------------------------------------------ allocation-free */

/* evaluate! for callers that may not allocate device memory.  No counterpart in the
 * reference: SplineGrids.jl allocates freely through KernelAbstractions.  Some hosts
 * cannot: code that runs under a fixed device-memory budget (a Julia task inside a
 * memory pool it must not grow, a plugin host that reserves the GPU's memory up
 * front) or a loop that must never block on the allocator.  They cannot create a
 * plan, whose scratch is allocated, but they can call this with the same descriptor,
 * derivative orders, control points, weights and eval as sg_evaluate; no plan and no
 * allocation is involved.
 *
 * The separable passes' intermediates live in a 64 MiB array that the library
 * declares statically on the device (every GPU that loads the library holds it until
 * the process exits); each intermediate, [n_samples of the axes already contracted,
 * n_basis of the others, nout (+1 for NURBS)] values, must fit in 32 MiB, otherwise
 * the call returns SG_ERR_UNSUPPORTED and names the size.  The first call on a device
 * looks the array's address up (cudaGetSymbolAddress) and should come before any
 * stream capture.  All calls share the one array: calls whose kernels can overlap on
 * the GPU (e.g. on different streams) race and must be serialized by the caller.
 * Sample indices are not range-checked on the host here (that needs a plan); out of
 * range indices are clamped by the kernels so that no access leaves the arrays. */
int sg_evaluate_noalloc(const sg_grid_desc *desc, const int32_t *derivative_order,
                        const void *control_points, const void *weights, void *eval,
                        sg_stream_t stream);

/* ------------------------------------------------------------------ least-squares fit */

/* Matrix-free LSQR (Paige & Saunders 1982) with its vectors and scalars on the device.
 * The reference fits a grid by wrapping it as a LinearMap (ext/SplineGridsLinearMapsExt.jl:
 * 5-52: forward = evaluate!(control_points); evaluate!(grid), adjoint =
 * evaluate_adjoint!(grid); evaluate_adjoint!(control_points)) and calling
 * IterativeSolvers.lsqr on it (test/test_LinearMapsExt.jl:14-61, docs fitting example).
 * The operator stays with the caller: between the solver's steps the caller applies
 * F = A V (m values) and G = A' U (n values) with the grid calls above.
 *
 * All six vectors are caller-owned device arrays of `dtype` (F32 or F64): U, F of length
 * m (= number of eval values), V, W, X, G of length n (= control-point unknowns).  One
 * solve, written out:
 *     sg_lsqr_start(h, b)           U = b, X = 0, beta = ||b||
 *     G = A' U ; sg_lsqr_after_adjoint(h)
 *     until done (sg_lsqr_info counts[2]):
 *         F = A V ; sg_lsqr_after_forward(h)
 *         G = A' U ; sg_lsqr_after_adjoint(h)
 * X then holds the solution.  Defaults of the reference's solver: atol = btol = sqrt(eps),
 * conlim = 1/sqrt(eps), maxiter = max(m, n), damp = 0.  A NaN or Inf in the recurrence
 * stops the solve with istop = -1.
 *
 * Graph form (one launch per solve, no host round trip): call sg_lsqr_capture_begin on a
 * stream, issue the prologue (start, adjoint, after_adjoint) on it, call
 * sg_lsqr_capture_body, issue one iteration (forward, after_forward, adjoint,
 * after_adjoint) on the returned body stream, then sg_lsqr_capture_end.  The body becomes
 * a device-side while loop that the solver ends when a stopping rule holds (or maxiter is
 * reached); sg_lsqr_launch runs the whole solve.  Pointers (b included) are baked into
 * the graph; the operator calls must allocate nothing while captured (create grid plans
 * before capturing). */
typedef struct sg_lsqr sg_lsqr;
int sg_lsqr_create(int32_t dtype, int64_t m, int64_t n, void *U, void *V, void *W, void *X,
                   void *F, void *G, double damp, double atol, double btol, double conlim,
                   int64_t maxiter, sg_lsqr **out);
int sg_lsqr_destroy(sg_lsqr *h);
int sg_lsqr_start(sg_lsqr *h, const void *b, sg_stream_t stream);
int sg_lsqr_after_forward(sg_lsqr *h, sg_stream_t stream);
int sg_lsqr_after_adjoint(sg_lsqr *h, sg_stream_t stream);
int sg_lsqr_capture_begin(sg_lsqr *h, sg_stream_t stream);
int sg_lsqr_capture_body(sg_lsqr *h, sg_stream_t stream, sg_stream_t *body);
int sg_lsqr_capture_end(sg_lsqr *h, sg_stream_t stream);
int sg_lsqr_launch(sg_lsqr *h, sg_stream_t stream);
/* Synchronizes `stream`; counts = {iterations, istop, done}, norms = {||A|| estimate,
 * cond(A) estimate, ||r||, ||A'r||, ||x||, ||b||}.  istop follows the paper: 0 x = 0 is
 * exact, 1 Ax = b to btol/atol, 2 least squares to atol, 3 cond(A) > conlim, 4-6 the same
 * at machine precision, 7 maxiter reached, -1 non-finite values. */
int sg_lsqr_info(sg_lsqr *h, sg_stream_t stream, int64_t *counts, double *norms);

/* ------------------------------------------------------------------ device selection */

/* Reductions and order-preserving compactions for local refinement, on the device:
 * error_informed_local_refinement! (src/control_points.jl:555-578: adjoint, sum over
 * outputs, threshold_factor * mean, findall, unique against the level's indices) and
 * deactivate_overwritten_control_points! (:584-680: Flag adjoint, findall of surviving
 * rows).  `workspace` holds sg_select_workspace_bytes(n) bytes for n elements (n = the
 * control points of the grid, or the rows).  Selections keep the reference's findall
 * order (column-major linear order) and are identical on every run. */
int64_t sg_select_workspace_bytes(int64_t n);

/* out[i] = sum over o of in[i + ncp*o] (in output order, in the array's type); *total
 * (device FP64) = sum over i of out[i], fixed-order. */
int sg_sum_outputs(int32_t dtype, int64_t ncp, int32_t nout, const void *in, void *out,
                   double *total, void *workspace, sg_stream_t stream);

/* Control points i of the grid cp_size[nin] with values[i] > threshold_factor * (*total) /
 * ncp (compared in FP64) that are not among exclude_idx ([n_exclude, nin], 1-based,
 * column-major), in linear order: out_idx[r + ncp*d] = their 1-based indices and, when
 * gather_src ([ncp, nout]) is given, out_vals[r + ncp*o] = gather_src[i + ncp*o].
 * Synchronizes `stream` and returns the count in *n_selected. */
int sg_select_above(int32_t dtype, int32_t nin, const int64_t *cp_size, int32_t nout,
                    const void *values, const double *total, double threshold_factor,
                    const int32_t *exclude_idx, int64_t n_exclude, const void *gather_src,
                    int32_t *out_idx, void *out_vals, int64_t *n_selected, void *workspace,
                    sg_stream_t stream);

/* Rows r of idx_in [n, nin] (Int32) and vals_in [n, nout] (dtype) with keep[r] > 0, in
 * order, into the first rows of idx_out / vals_out (same [n, .] column-major layout).
 * Synchronizes `stream` and returns the count in *n_kept. */
int sg_select_rows(int32_t dtype, int64_t n, const double *keep, int32_t nin,
                   const int32_t *idx_in, int32_t nout, const void *vals_in, int32_t *idx_out,
                   void *vals_out, int64_t *n_kept, void *workspace, sg_stream_t stream);

/* ------------------------------------------------------------------ refinement matrices */

/* The refinement matrix of inserting n_insert knots in order into the expanded knot
 * vector knots_all_old (n_knots_old values, device), built on the device in one launch:
 * the composition R = R_n ... R_1 of the single-knot matrices
 * (build_refinement_matrix_kernel, src/refinement.jl:3-36) by the banded product
 * (src/refinement_matrix.jl:184-327), which refine(::SplineDimension) runs one knot at
 * a time on the host loop (src/refinement.jl:275-279).  knot_span_index[q] (device,
 * 1-based) is knot q's span in the knot vector at its insertion: the number of knots
 * below it.  Outputs in the RefinementMatrix layout, rows = n_knots_old - degree - 1 +
 * n_insert: row_pointer, column_start (1-based, [rows]) and nzval (capacity rows *
 * (degree + 2)); *nnz (host) = stored values.  Bit-identical to composing the products
 * one by one in the reference's operation order.  Synchronizes `stream`; returns
 * SG_ERR_DEVICE_CHECK if a row's band would exceed degree + 2 values. */
int64_t sg_refine_matrix_workspace_bytes(int32_t dtype, int32_t degree, int64_t n_knots_old,
                                         int64_t n_insert);
int sg_refine_matrix(int32_t dtype, int32_t degree, const void *knots_all_old,
                     int64_t n_knots_old, int64_t n_insert, const void *knots_new,
                     const int32_t *knot_span_index, int32_t *row_pointer, int32_t *column_start,
                     void *nzval, int64_t *nnz, void *workspace, sg_stream_t stream);

/* ------------------------------------------------------------------ fit loop stages */

/* The loss and update stages of a gradient-descent fit, the user loop of the reference's
 * optimisation examples (docs/src/examples_optics.md:184-191: evaluate! of (0,0), (1,0),
 * (0,1), a loss on the evals, its gradient through evaluate_adjoint! by Enzyme, an
 * optimiser step).  Between sg_evaluate(_multi) and sg_evaluate_adjoint, over fixed
 * device arrays, so that the whole step can be captured into one CUDA graph:
 *   sg_fit_loss:   cotangent_t = w_t (eval_t - target_t) for every term t (n_values[t]
 *                  values each; weights NULL = all 1), and
 *                  loss = sum_t w_t / 2 sum_i (eval_t[i] - target_t[i])^2 as a fixed-order
 *                  FP64 sum (bitwise reproducible), kept on the device;
 *   sg_fit_update: params_u -= step * (sum of its grad_counts[u] gradient arrays, taken in
 *                  order from `grads`) for every parameter array u (param_sizes[u] values).
 * dtype SG_F32 or SG_F64 (all arrays).  Arrays and sizes are fixed at creation.
 * sg_fit_losses synchronizes `stream` and returns the latest loss, the number of loss
 * stages run, and (history != NULL) up to `capacity` of the last 1024 losses, oldest
 * first. */
typedef struct sg_fit_plan sg_fit_plan;
int sg_fit_plan_create(int32_t dtype, int32_t n_terms, void *const *evals,
                       const void *const *targets, void *const *cotangents,
                       const int64_t *n_values, const double *weights, int32_t n_params,
                       void *const *params, const int64_t *param_sizes,
                       const int32_t *grad_counts, void *const *grads, sg_fit_plan **out);
int sg_fit_plan_destroy(sg_fit_plan *p);
int sg_fit_loss(sg_fit_plan *p, sg_stream_t stream);
int sg_fit_update(sg_fit_plan *p, double step, sg_stream_t stream);
int sg_fit_losses(sg_fit_plan *p, sg_stream_t stream, double *latest, int64_t *count,
                  double *history, int64_t capacity);

/* ------------------------------------------------------------------ test hooks */

/* For tests of the failure paths only; the defaults are restored by passing -1 / 0.
 * sg_test_fail_allocations: every device allocation of a plan or handle after the next
 *   `after` ones fails with SG_ERR_OUT_OF_MEMORY (after < 0: none fails);
 *   sg_test_live_allocations counts the live ones, to show that a failed create leaks
 *   nothing.
 * sg_test_set_wait_limits: the poll limit of the batch pass queue's dependency waits and
 *   the SM-cycle budget of the fused adjoint's stage waits (<= 0: the defaults, about
 *   half a second and one second).
 * sg_test_block_waits: batch_dependency != 0 makes every pass-queue dependency ask for
 *   one tile more than its pass has (it can never complete); fused_first_stage != 0
 *   makes the fused adjoint's producer withhold its arrival on each CTA's first stage.
 *   Either way the bounded waits run out, the kernels return, and sg_batch_check /
 *   sg_grid_plan_check report SG_ERR_TIMEOUT. */
int sg_test_fail_allocations(int64_t after);
int64_t sg_test_live_allocations(void);
int sg_test_set_wait_limits(int64_t batch_spin_limit, int64_t mbar_wait_cycles);
int sg_test_block_waits(int32_t batch_dependency, int32_t fused_first_stage);

#ifdef __cplusplus
}
#endif

#endif /* SPLINEGRIDS_B200_H */
