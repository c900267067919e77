/*
 * gbg_transfer.h -- C ABI of the GB300 (sm_103a) particle gather/scatter library.
 *
 * This library replaces the spline transfer path of GBGPeriodicFields.jl
 * (src/Interpolation.jl, src/Points.jl, and the device storage of src/Fields.jl).
 * Every entry point is extern "C" with plain pointers and sizes, returns a status
 * code, never throws and never aborts.  A Julia facade binds these with ccall and
 * maps the status codes to the reference's exceptions (ArgumentError,
 * DimensionMismatch).
 *
 * Conventions (the reference's, 0-based here):
 *   - arrays are column-major:
 *       field      (Nx, Ny, Nz, ncomp):  f[x + Nx*y + Nx*Ny*z + N*c], N = Nx*Ny*Nz
 *       positions  (M, 3):               pos[p + M*d]
 *       values     (M, ncomp):           v[p + M*c]
 *     ncomp = 3^R for a tensor field of order R (R = 0 scalar, 1 vector, ...); a
 *     tensor fibre is itself column-major (Interpolation.jl:1038-1048).
 *   - all array pointers are DEVICE pointers unless stated otherwise;
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *     Calls are stream-ordered and asynchronous; the reference's transfers are
 *     synchronous, so a facade synchronizes the stream before returning;
 *   - `device_status` (optional, may be NULL) is a device int32 that kernels OR
 *     GBG_DEV_* bits into.  Device code never traps: invalid input found on the
 *     device (a non-finite position, an out-of-range traversal entry) is reported
 *     here and the affected point is skipped or yields NaN.
 */
#ifndef GBG_TRANSFER_H
#define GBG_TRANSFER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBG_ABI_VERSION 1

typedef int32_t gbg_status;
#define GBG_OK 0
#define GBG_EARG 1          /* ArgumentError: bad scheme, tensor order, precision, order ... */
#define GBG_EDIM 2          /* DimensionMismatch: point counts differ */
#define GBG_ENOMEM 3        /* device allocation failed or workspace too small */
#define GBG_ECUDA 4         /* a CUDA runtime call failed */
#define GBG_ENONFINITE 5    /* a non-finite or out-of-range position reached the locate step */
#define GBG_ETIMEOUT 6      /* a bounded wait gave up */
#define GBG_EUNSUPPORTED 7  /* outside the sizes this build handles (stated per entry point) */
#define GBG_EBUSY 8         /* admission refused (serving) */
#define GBG_ETRAVERSAL 9    /* a traversal order is not a permutation of 1:M */

typedef int32_t gbg_dtype;
#define GBG_F32 1
#define GBG_F64 2

/* Bits written to *device_status by kernels. */
#define GBG_DEV_NONFINITE 1
#define GBG_DEV_TRAVERSAL 2
#define GBG_DEV_TIMEOUT 4 /* a bounded wait on a shared-memory copy gave up */

/* Grid3D (Fields.jl:165-200).  spacing is stored, as in the reference, and must equal
 * domain ./ n in the transfer's element type. */
typedef struct {
  int64_t n[3];
  double domain[3];
  double spacing[3];
  double origin[3];
} gbg_grid;

#define GBG_MAX_NODES 16
#define GBG_MAX_POWERS 32
#define GBG_SCHEME_CUSTOM 0
#define GBG_SCHEME_LALESCU 1
#define GBG_SCHEME_LAGRANGE 2

/* A local spline scheme (Interpolation.jl:227-312): stencil_width = N2 = 2n+2 nodes
 * per axis at offsets -n..n+1, weight polynomials of num_powers = M2 coefficients.
 * coefficients[q + N2*r] is the t^r coefficient of node q, in Float64. */
typedef struct {
  int32_t kind;
  int32_t stencil_width;
  int32_t smoothness; /* LalescuSpline's m; -1 for the others */
  int32_t num_powers;
  double coefficients[GBG_MAX_NODES * GBG_MAX_POWERS];
} gbg_scheme;

/* ---------------------------------------------------------------- general */

/* ABI version (GBG_ABI_VERSION). */
int32_t gbg_abi_version(void);
/* Static text for a status code. */
const char *gbg_status_string(gbg_status status);
/* The calling host thread's message for its last failed call ("" if none). */
const char *gbg_last_error(void);
/* Number of kernels this library has launched in this process (all threads). */
uint64_t gbg_kernel_launches(void);
/* Measurement hook (no counterpart in the reference): with two CUDA events (cudaEvent_t,
 * created with timing), every later transfer call from this host thread records the first
 * just before and the second just after its main kernel (the gather kernel, or the brick
 * accumulation kernel of a scatter), on the call's stream, so that a benchmark can time
 * that kernel alone.  NULL, NULL switches it off. */
gbg_status gbg_set_kernel_timing_events(void *start_event, void *stop_event);

/* ---------------------------------------------------------------- schemes */

/* LalescuSpline(stencil_width; smoothness) -- Interpolation.jl:244-258 (with
 * _stencil_neighbours 236-241, _fornberg 326-354, _hermite_weight_matrix 367-392).
 * smoothness < 0 selects the default stencil_width/2 - 1.  CatmullRom is (4, 1)
 * (Interpolation.jl:424).  GBG_EARG for an odd or < 2 width or m outside 0..2n. */
gbg_status gbg_scheme_lalescu(int32_t stencil_width, int32_t smoothness, gbg_scheme *out);
/* LagrangeSpline(stencil_width) -- Interpolation.jl:293-306 (_lagrange_weight_matrix
 * 403-415). */
gbg_status gbg_scheme_lagrange(int32_t stencil_width, gbg_scheme *out);
/* A scheme from caller coefficients (N2 x M2, column-major, Float64): what a facade
 * passes when it holds the reference's own SMatrix (spline_coefficients, 311-312). */
gbg_status gbg_scheme_custom(int32_t stencil_width, int32_t num_powers,
                             const double *host_coefficients, gbg_scheme *out);
/* Host helper: the N2 per-axis weights at t (Interpolation.jl:440-446), Float64. */
gbg_status gbg_axis_weights(const gbg_scheme *scheme, double t, double *host_weights);

/* ---------------------------------------------------- drop-in transfers */

/* interpolate! -- Interpolation.jl:1181-1198 (kernel 1007-1052).  Gathers the
 * ncomp-component field at the M points into out (M, ncomp).  field, positions and
 * out share dtype (the reference refuses mixed precision, 1125-1138).  traversal is
 * NULL or a 1-based permutation of 1:M (PointTraversalOrder indices, 618-627); it
 * changes only the visiting order and the result is bitwise the same with or
 * without it.  M = 0 is legal. */
gbg_status gbg_interpolate(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp,
                           const void *field, const void *positions, int64_t npoints,
                           const int32_t *traversal, const gbg_scheme *scheme, void *out,
                           int32_t *device_status, void *stream);

/* anterpolate! -- Interpolation.jl:1299-1323 (kernel 1063-1106, prescale 1309-1313):
 * field = alpha * W^T q + beta * field, with beta == 0 overwriting (NaN-safe).
 * Deterministic: the result is bitwise identical run to run and independent of the
 * traversal (points are sorted by brick and cell on the device and every brick sums its
 * nodes' contributions as 64-bit fixed-point integers, whose sum does not depend on the
 * order of the additions; no float atomics).  workspace: device scratch
 * of at least gbg_anterpolate_workspace_size bytes, or NULL (the library then takes
 * stream-ordered scratch with cudaMallocAsync and releases it before returning). */
gbg_status gbg_anterpolate(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp, void *field,
                           const void *positions, int64_t npoints, const void *quantities,
                           const int32_t *traversal, const gbg_scheme *scheme, double alpha,
                           double beta, void *workspace, size_t workspace_bytes,
                           int32_t *device_status, void *stream);
gbg_status gbg_anterpolate_workspace_size(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp,
                                          int64_t npoints, const gbg_scheme *scheme,
                                          size_t *bytes);

/* anterpolate! for callers that cannot allocate device memory.  This entry point has no
 * counterpart in the reference.  It computes exactly what gbg_anterpolate computes, but
 * its scratch is a fixed array compiled into this library (GBG_NOALLOC_SCRATCH_BYTES,
 * 64 MiB, held on every device that loads the library until the process exits), so it
 * calls no cudaMalloc, cudaFree or other allocating routine.  It exists for callers
 * whose device memory is not theirs to allocate mid-run: a host that reserves the
 * GPU's memory up front through its own pool, and a caller held to the reference's
 * in-place contract that anterpolate! allocates nothing (test/allocations.jl:335-361).
 * A problem whose scratch (gbg_anterpolate_workspace_size) exceeds the array is
 * refused with GBG_EUNSUPPORTED.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the context current at the call, so the address is never
 * stale after a device reset; the first call on a device may load the library's device
 * image, so make it before any stream capture.  Every call shares the one array: calls
 * that overlap on the GPU (different streams, or different host threads, on the same
 * device) race and must be serialized by the caller. */
#define GBG_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
gbg_status gbg_anterpolate_noalloc(const gbg_grid *grid, gbg_dtype dtype, int32_t ncomp,
                                   void *field, const void *positions, int64_t npoints,
                                   const void *quantities, const gbg_scheme *scheme,
                                   double alpha, double beta, int32_t *device_status,
                                   void *stream);

/* point_traversal_order / point_traversal_order! -- Interpolation.jl:816-833 and
 * 953-980 (keys 645-661 with the saturating _tile_index 636-642).  Writes a 1-based
 * permutation into order (M int32) grouping points by tile_size^3-cell tiles.  The
 * device sort is stable, so within a tile points keep their index order: the result
 * is deterministic and is one of the orders the reference can return.
 * GBG_EUNSUPPORTED if the tile count reaches 2^32. */
gbg_status gbg_point_traversal_order(const gbg_grid *grid, gbg_dtype dtype,
                                     const void *positions, int64_t npoints, int64_t tile_size,
                                     int32_t *order, void *workspace, size_t workspace_bytes,
                                     void *stream);
gbg_status gbg_point_traversal_order_workspace_size(const gbg_grid *grid, int64_t npoints,
                                                    int64_t tile_size, size_t *bytes);

/* PointTraversalOrder validation -- Interpolation.jl:560-589.  Synchronous: returns
 * GBG_OK if order is a permutation of 1:M, GBG_ETRAVERSAL otherwise, and reports the
 * extrema and the number of distinct points visited through the host pointers. */
gbg_status gbg_validate_traversal(const int32_t *order, int64_t npoints, int64_t *host_low,
                                  int64_t *host_high, int64_t *host_visited, void *stream);

/* ------------------------------------------- resident storage and binned transfers
 *
 * The device storage of a field (replacing Fields.jl's column-major (Nx,Ny,Nz,3^R)
 * CuArray, 922-974) and a device cell-binned sort of a point set (replacing
 * point_traversal_order, Interpolation.jl:519-980) that the staged gather and the
 * deterministic scatter both consume.  Handles are opaque; every handle belongs to
 * the device that was current when it was created. */

typedef struct gbg_field_s *gbg_field;
typedef struct gbg_bins_s *gbg_bins;

/* A field of ncomp components on grid, stored as storage_dtype with the components
 * of a node adjacent (padded to 16 bytes) and a periodic ghost layer wide enough for
 * stencils up to max_stencil_width nodes, so a brick of cells plus its halo is one
 * contiguous box.  Allocates on the current device. */
gbg_status gbg_field_create(const gbg_grid *grid, int32_t ncomp, gbg_dtype storage_dtype,
                            int32_t max_stencil_width, gbg_field *out);
gbg_status gbg_field_destroy(gbg_field field);
/* Copies a reference-layout (Nx,Ny,Nz,ncomp) array of src_dtype into the storage,
 * converting, and fills the ghost layer. */
gbg_status gbg_field_import(gbg_field field, gbg_dtype src_dtype, const void *src, void *stream);
/* Copies the storage out to a reference-layout array of dst_dtype. */
gbg_status gbg_field_export(gbg_field field, gbg_dtype dst_dtype, void *dst, void *stream);
/* Device bytes the storage holds. */
gbg_status gbg_field_bytes(gbg_field field, size_t *bytes);

/* Bins for up to max_points points on grid, grouped by bricks of brick[0] x brick[1] x
 * brick[2] cells (NULL selects 11 x 8 x 8, and an edge of 0 that edge's default; each
 * edge 1..64).  Allocates on the current
 * device. */
gbg_status gbg_bins_create(const gbg_grid *grid, int64_t max_points, const int32_t *brick,
                           gbg_bins *out);
gbg_status gbg_bins_destroy(gbg_bins bins);
/* ---------------------------------------------------------- displacement
 * Points.jl:1382-1440 (displace!) and 1481-1490 (wrap!): per coordinate
 * dst = ((src + c_1 v_1) + c_2 v_2) + ... in the positions' type, every product and sum
 * rounded separately as the reference's broadcast does, then, with a grid (or wrap != 0),
 * reduced to [origin, origin + domain) by _wrap_coordinate (Points.jl:1245-1249: the
 * excluded endpoint folded to the origin, non-finite coordinates left non-finite).
 * Positions and the nterms sections are device (M, 3) column-major arrays of dtype; the
 * coefficients are host doubles converted to dtype; dst may equal src.  nterms = 0 with a
 * grid is wrap!. */
#define GBG_MAX_TERMS 32
gbg_status gbg_points_displace(const gbg_grid *grid /* NULL: no wrap */, gbg_dtype dtype, void *dst, const void *src,
                               int64_t npoints, int32_t nterms, const double *coefficients,
                               const void *const *sections, void *stream);
/* The displacement fused with the bins build: the moved (and, with wrap != 0, wrapped)
 * positions are written to dst and binned in the same pass over the points, which keeps a
 * particle loop's points binned from step to step without a second read of the positions. */
gbg_status gbg_bins_build_displaced(gbg_bins bins, gbg_dtype dtype, void *dst, const void *src, int64_t npoints,
                                    int32_t nterms, const double *coefficients, const void *const *sections,
                                    int32_t wrap, int32_t *device_status, void *stream);
/* Copies an (M, ncols) column-major array into the bins' sorted order
 * (dst[s + M*c] = src[perm[s] + M*c]); applied to the positions and every per-point array
 * it keeps the particle state in binned order.  src and dst must differ. */
gbg_status gbg_bins_permute(gbg_bins bins, gbg_dtype dtype, int32_t ncols, const void *src, void *dst,
                            void *stream);
/* Threads per CTA of the binned gather (0 = default, 128, 256 or 512) and scatter
 * (0 = default, 64, 128 or 256) launched on these bins: the autotuner's knobs beside
 * the brick edges.  Each CTA works through whole bricks; the grid is sized from the
 * occupancy the choice allows.  No counterpart in the reference. */
gbg_status gbg_bins_set_launch(gbg_bins bins, int32_t gather_threads, int32_t scatter_threads);
/* Compensated summation in gbg_anterpolate_binned on these bins: 1 (the default) sums each
 * node in FP32 over every chunk of at most 1024 of its brick region's points and folds the
 * chunk sums into a running (sum, correction) pair by TwoSum (the corrections live in a
 * per-CTA slot of the bins' device block); 0 carries one plain FP32 running sum.  A region
 * that fits in one chunk is summed the same way either way.  No counterpart in the
 * reference, whose scatter sums in its field's own precision. */
gbg_status gbg_bins_set_compensated(gbg_bins bins, int32_t compensated);
/* Regions of the binned scatter for point sets sparse on their grid (fewer than four points
 * a brick): 1 (the default) lets a brick take its region's points from the point lists of
 * its 27 neighbouring bricks when they hold few enough; 0 always builds the region's
 * per-cell tables.  Both give the same points in the same order, so the same bits; the
 * switch exists for tests and tuning.  No counterpart in the reference. */
gbg_status gbg_bins_set_sparse_regions(gbg_bins bins, int32_t allow);
/* Polls of a staged tile's mbarrier before gbg_interpolate_binned gives up on it (0 = the
 * default, 2^22 suspending polls; a smaller limit polls without suspending): the wait then
 * sets GBG_DEV_TIMEOUT, the CTA lets its copies land (always with the full limit) and
 * returns, leaving that tile's points unwritten.  A failure-path control with no
 * counterpart in the reference; a tiny limit makes the wait run out on purpose, which is
 * how the timeout path is tested. */
gbg_status gbg_bins_set_wait_limit(gbg_bins bins, uint32_t polls);
/* Bins the points: each position is wrapped periodically and split into a cell index
 * and a fractional offset in the positions' own precision (FP64 positions keep FP64
 * for this step), then the points are stably sorted by brick and cell on the device.
 * A non-finite position sets GBG_DEV_NONFINITE and is placed in cell 0 with NaN
 * weights. */
gbg_status gbg_bins_build(gbg_bins bins, gbg_dtype pos_dtype, const void *positions,
                          int64_t npoints, int32_t *device_status, void *stream);
/* Many bins built in one call: count bins, each from its own positions (dtype, pointer,
 * count), as gbg_bins_build would build them one after another.  Independent bins build
 * at the same time on the library's side streams, forked from and joined back to stream
 * (inside a stream capture: parallel branches of the graph); the same bins twice build in
 * call order.  The side streams are made by gbg_bins_create and gbg_batch_create.  No
 * counterpart in the reference. */
gbg_status gbg_bins_build_batch(const gbg_bins *bins, const gbg_dtype *dtypes, const void *const *positions,
                                const int64_t *npoints, int32_t count, int32_t *device_status, void *stream);
/* The binned order as a 1-based traversal order (point_traversal_order's output). */
gbg_status gbg_bins_order(gbg_bins bins, int32_t *order, void *stream);

/* Gather of a resident field at binned points into out (M, ncomp) of out_dtype, in the
 * points' own order.  scheme width must not exceed the field's max_stencil_width.  A
 * bounded wait on a staged tile that gives up sets GBG_DEV_TIMEOUT in device_status (may
 * be NULL) and leaves that tile's points unwritten. */
gbg_status gbg_interpolate_binned(gbg_field field, gbg_bins bins, const gbg_scheme *scheme,
                                  gbg_dtype out_dtype, void *out, int32_t *device_status, void *stream);
/* Deterministic scatter of q (M, ncomp) of q_dtype at binned points into a resident
 * field: field = alpha * W^T q + beta * field.  No atomics: each node's sum is formed
 * by one thread in a fixed order (the node's rows of cells, within a row the points in
 * binned order), so the result is bitwise reproducible and independent of the launch
 * shape; the ghost layer is refreshed.  A non-finite quantity sets GBG_DEV_NONFINITE in
 * device_status (may be NULL). */
gbg_status gbg_anterpolate_binned(gbg_field field, gbg_bins bins, const gbg_scheme *scheme,
                                  gbg_dtype q_dtype, const void *q, double alpha, double beta,
                                  int32_t *device_status, void *stream);

/* ------------------------------------------------------------ batched form
 *
 * Many independent instances of uneven sizes (fields of different grids and component
 * counts, point sets of different sizes, mixed stencil widths) run as ONE persistent
 * gather launch and ONE persistent scatter launch: every (instance, brick) is a unit of
 * work that the CTAs take from a device counter, largest instances first.  Instances of
 * 1024 points or more run through the single-instance kernels of gbg_interpolate_binned /
 * gbg_anterpolate_binned instead, which are faster for them (same results: both sums are
 * formed in an order fixed by the points); every gather still runs before any scatter.
 * The batch holds device copies of each pooled instance's geometry, scheme and TMA
 * descriptor, so gbg_batch_run issues only stream operations and can be captured in a
 * CUDA graph together with the gbg_bins_build calls that precede it. */
typedef struct gbg_batch_s *gbg_batch;
typedef struct {
  gbg_field field;    /* gathered from (FP32 resident storage) */
  gbg_bins bins;      /* the instance's binned points */
  gbg_scheme scheme;  /* stencil of 2, 4, 6 or 8 nodes with num_powers == stencil_width */
  float *out;         /* gather output, (M, ncomp) in the points' order, or NULL */
  gbg_field dest;     /* scatter destination (same grid and components as field), or NULL */
  const float *q;     /* scatter quantities, (M, ncomp) in the points' order */
  double alpha, beta; /* dest = alpha * W^T q + beta * dest */
} gbg_batch_item;
gbg_status gbg_batch_create(const gbg_batch_item *items, int32_t count, gbg_batch *out);
/* Runs the batch on stream: the scatters' quantity preparation, one gather launch, one
 * scatter launch, and the ghost refresh of every destination. */
gbg_status gbg_batch_run(gbg_batch batch, int32_t *device_status, void *stream);
gbg_status gbg_batch_destroy(gbg_batch batch);

/* ------------------------------------------------------------------ serving loop
 *
 * No counterpart in the reference, which is a library called in-process with no request
 * loop.  A server keeps resident fields on the device and runs a native progress thread
 * over `slots` CUDA streams.  Requests -- a gather from, or a scatter into, a resident
 * field at device-resident positions -- queue in arrival order.  Whenever a slot is free,
 * the thread takes the longest run of queued requests from the head that (1) numbers at
 * most max_batch, (2) fits, with the bins it needs, in the memory budget still free, and
 * (3) touches no field twice in a way the batch kernels would race on (a second scatter
 * into a field, or a gather from a field the run already scatters into), builds each
 * request's bins on the slot's stream and runs the run as one batch (gbg_batch_run).
 * Requests that arrive while others are on the device are admitted as slots and memory
 * free up, and the runs of different slots overlap on the device.  Requests on the same
 * field keep their arrival order -- a gather sees every earlier scatter into its field
 * and no later one -- through stream events, without blocking the host.  The thread
 * learns of completion by polling events; a run whose device work passes
 * timeout_seconds is reported as GBG_ETIMEOUT, and its memory is held until the device
 * has finished with it.  Fault injection (gbg_server_inject) acts on the host only.
 * While requests on a field are queued or in flight, the caller makes no other call on
 * that field. */
typedef struct gbg_server_s *gbg_server;
typedef struct {
  int32_t slots;            /* runs in flight at once, one stream each, 1..64 */
  int32_t max_batch;        /* requests per run, 1..256 */
  int32_t brick[3];         /* bins' brick edges; 0 selects the default edge */
  int32_t reserved;
  size_t hbm_budget_bytes;  /* device memory the server may hold for requests; 0 = half the free memory */
  double timeout_seconds;   /* deadline of one run's device work, > 0 */
} gbg_server_config;

#define GBG_REQ_INTERPOLATE 1
#define GBG_REQ_ANTERPOLATE 2
typedef struct {
  int32_t kind;           /* GBG_REQ_INTERPOLATE or GBG_REQ_ANTERPOLATE */
  gbg_dtype pos_dtype;    /* GBG_F32 or GBG_F64 positions */
  gbg_field field;        /* gathered from (interpolate) or scattered into (anterpolate) */
  gbg_scheme scheme;      /* 2, 4, 6 or 8 nodes with num_powers == stencil_width */
  const void *positions;  /* device, (npoints, 3) column-major; kept alive until completion */
  int64_t npoints;
  float *out;             /* interpolate: device (npoints, ncomp) column-major FP32 */
  const float *q;         /* anterpolate: device (npoints, ncomp) column-major FP32 */
  double alpha, beta;     /* anterpolate: field = alpha * W^T q + beta * field */
  void *ready_event;      /* a cudaEvent_t the run waits for before reading the request's
                             arrays (recorded by the caller after producing them and not
                             re-recorded until the request completes), or NULL when the
                             arrays are ready at submission */
} gbg_request;

typedef struct {
  int64_t submitted, completed, failed, queued, in_flight, runs;
  int64_t points;                  /* points of the completed requests */
  double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> observed completion */
  double first_submit_s, last_done_s;      /* on the server's steady clock */
  size_t hbm_in_use, hbm_peak, hbm_budget;
} gbg_server_counters;

gbg_status gbg_server_create(const gbg_server_config *config, gbg_server *out);
/* Queues a request and returns its ticket.  A request whose bins alone exceed the
 * budget is refused here (GBG_EBUSY); malformed requests return GBG_EARG. */
gbg_status gbg_server_submit(gbg_server server, const gbg_request *request, int64_t *ticket);
/* Waits up to timeout_seconds for a ticket.  Returns GBG_OK with the request's own
 * status in *result (GBG_OK, GBG_ENONFINITE for a non-finite position, GBG_ETIMEOUT,
 * GBG_ENOMEM, GBG_ECUDA), or GBG_ETIMEOUT if the request is still pending.  A ticket
 * can be waited for once. */
gbg_status gbg_server_wait(gbg_server server, int64_t ticket, double timeout_seconds, gbg_status *result);
/* Waits up to timeout_seconds until nothing is queued or in flight. */
gbg_status gbg_server_drain(gbg_server server, double timeout_seconds);
/* Counters and latency percentiles since creation or the last reset (reset != 0 clears
 * them after reading). */
gbg_status gbg_server_stats(gbg_server server, int32_t reset, gbg_server_counters *out);
#define GBG_FAULT_ALLOC 1    /* the next `count` request allocations fail (GBG_ENOMEM) */
#define GBG_FAULT_DEADLINE 2 /* the next `count` runs get a deadline already passed (GBG_ETIMEOUT) */
gbg_status gbg_server_inject(gbg_server server, int32_t fault, int32_t count);
/* Drains (bounded by the timeout given at creation), stops the thread and frees. */
gbg_status gbg_server_destroy(gbg_server server);
/* The admission rule on its own, for planning: of n queued requests (kinds, fields as
 * opaque ids, device bytes), how many from the head form the next run given free_bytes
 * and max_batch.  0 means the head request waits for memory. */
gbg_status gbg_server_plan(const int32_t *kinds, const uint64_t *fields, const size_t *bytes, int32_t n,
                           size_t free_bytes, int32_t max_batch, int32_t *run_length);

/* ------------------------------------------------------------- NUFFT window transfers
 *
 * The per-point steps of the reference's fast spectral transfer (Interpolation.jl:1611-2070,
 * NUFFT): a gather from, and a spread onto, the oversampled (sigma*N) physical grid with
 * the exponential-of-semicircle window psi(s) = exp(beta*(sqrt(1 - (2s/W)^2) - 1)) over W
 * nodes per axis (_es_weights, 1638-1645; odd widths follow the nearer node, 1634-1635).
 * `fine` is the oversampled grid (its origin and spacing locate the points); fields on
 * it are (n0, n1, n2, ncomp) column-major in dtype.  Widths 1..16 (the reference derives
 * W = max(4, ceil(-log10(tolerance)) + 2), 16 at tolerance 1e-14); GBG_EUNSUPPORTED above.
 * The FFT of the oversampled grid, the exchange of modes with the reference grid and the
 * deconvolution are whole-array steps done by the caller (cuFFT). */

/* Host helper: the per-axis deconvolution factors 1/psi_hat(omega) of one axis of the
 * reference grid -- _nufft_deconvolution / _es_window_transform (Interpolation.jl:1652-1705):
 * for stored index i (frequency i on the half axis, else i or i - n), omega =
 * 2*pi*frequency/(oversampling*n), psi_hat by the 256-interval trapezoidal rule in theta
 * (z = sin theta), computed in dtype; an even axis's Nyquist entry is 0.  host_out holds
 * n/2+1 (is_half) or n values. */
gbg_status gbg_nufft_deconvolution_axis(int64_t n, int32_t is_half, int32_t oversampling, int32_t width,
                                        double beta, gbg_dtype dtype, double *host_out);
/* Device bytes of the gather's workspace: the points' tiles, ranks, places and first
 * stencil nodes (about 24 bytes per point) and the tile counts. */
gbg_status gbg_nufft_interp_workspace_size(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, int64_t npoints,
                                           int32_t width, size_t *bytes);
/* Type 2 window gather -- _nufft_gather_kernel! (Interpolation.jl:1864-1914):
 * out[p + M*c] = sum over the W^3 stencil of psi_x psi_y psi_z field[node, c].  FP32:
 * the points are binned by 8^3-node tiles of the oversampled grid and each tile's region is
 * staged in shared memory; FP64: a thread per point (the workspace is then unused).  A
 * non-finite position sets GBG_DEV_NONFINITE and yields NaN.  workspace: 256-byte aligned. */
gbg_status gbg_nufft_interp(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, const void *field,
                            const void *positions, int64_t npoints, const int32_t *traversal, int32_t width,
                            double beta, void *out, void *workspace, size_t workspace_bytes,
                            int32_t *device_status, void *stream);
/* Device bytes of the spread's workspace: int64 node sums, the points' tiles, ranks and
 * window weights (about npf*ncomp*8 + npoints*(24 + 3*width*sizeof(dtype)) bytes). */
gbg_status gbg_nufft_spread_workspace_size(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, int64_t npoints,
                                           int32_t width, size_t *bytes);
/* Type 1 window spread -- _nufft_spread_kernel! (Interpolation.jl:1919-1950): field (on
 * the oversampled grid, overwritten) = sum over points of ((psi_y psi_z) psi_x) q.
 * Deterministic where the reference adds floats atomically: each contribution is rounded
 * to 64-bit fixed point at one scale per call (2^k, M*max|q| < 2^(61-k)) and added as an
 * integer, so the result is the same bits whatever the thread order or traversal; its
 * absolute resolution is M*max|q|*2^-62 per contribution.  The points are binned by 8^3-
 * node tiles of the oversampled grid and each tile's sums are formed in shared memory
 * before one global add per node.  A non-finite quantity makes the whole field NaN (the
 * FFT spreads it over every mode in the reference too).  workspace: 256-byte aligned. */
gbg_status gbg_nufft_spread(const gbg_grid *fine, gbg_dtype dtype, int32_t ncomp, void *field,
                            const void *positions, int64_t npoints, const void *quantities,
                            const int32_t *traversal, int32_t width, double beta, void *workspace,
                            size_t workspace_bytes, int32_t *device_status, void *stream);

#ifdef __cplusplus
}
#endif
#endif
