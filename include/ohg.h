/* omega_h_gb300: GB300 (sm_103a) implementation of the per-pass core of
 * Omega_h::adapt() — metric edge lengths, cavity qualities for refine,
 * coarsen and 3D edge swap, the independent-set selection and the
 * adjacency rebuild — behind a C ABI over device pointers.
 *
 * Every function returns an ohg status code (OHG_OK on success); the
 * message of the last failure on the calling thread is ohg_last_error().
 * Arrays named *_dev are device pointers owned by the caller; sizes are in
 * elements.  Integer formats follow the reference: LO = int32, GO = int64,
 * Real = double, alignment codes = int8 laid out as
 * which_down<<3 | rotation<<1 | flip (src/Omega_h_align.hpp:44-51).
 * Calls on one context are ordered on that context's stream and return after
 * the device work finished.
 */
#ifndef OHG_H
#define OHG_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OHG_OK = 0,
  OHG_ERR_CUDA = 1,          /* a CUDA runtime call failed */
  OHG_ERR_BOUNDS = 2,        /* an index outside its array */
  OHG_ERR_LOOP_TOO_BIG = 3,  /* an edge ring larger than a kernel supports */
  OHG_ERR_NO_MATCH = 4,      /* reflect_down found no unique matching entity */
  OHG_ERR_TIMEOUT = 5,       /* an iterative selection did not converge */
  OHG_ERR_OOM = 6,           /* device allocation failed */
  OHG_ERR_ADMISSION = 7,     /* request exceeds the admission budget */
  OHG_ERR_INVALID = 8,       /* bad argument */
  OHG_ERR_NUMERIC = 9,       /* degenerate metric eigen-decomposition */
  OHG_ERR_TOPOLOGY = 10      /* mesh topology inconsistent with the operation */
};

typedef struct ohg_context ohg_context;
typedef struct ohg_mesh ohg_mesh;

/* The AdaptOpts fields used by one pass (src/Omega_h_adapt.hpp:50-77). */
typedef struct ohg_adapt_opts {
  double min_length_desired;
  double max_length_desired;
  double max_length_allowed;
  double min_quality_allowed;
  double min_quality_desired;
  int nsliver_layers;
} ohg_adapt_opts;

typedef struct ohg_pass_stats {
  int did_refine, did_coarsen, did_swap;
  int nelems_in, nelems_out;
  int refine_keys, coarsen_keys, swap_keys;
  int indset_rounds;
  double min_quality;
  float ms_refine, ms_coarsen, ms_swap;
} ohg_pass_stats;

/* Outcome of ohg_adapt: whether the mesh needed work, how many times each
 * operator changed it, and whether min_quality_desired was reached. */
typedef struct ohg_adapt_result {
  int did, quality_satisfied;
  int refines, coarsens, swaps, sliver_coarsens, length_rounds;
} ohg_adapt_result;

const char* ohg_last_error(void);

/* ---- context: one device, one stream, one stream-ordered memory pool ---- */
int ohg_context_create(int device, ohg_context** out);
int ohg_context_destroy(ohg_context* ctx);
/* number of kernels this library has launched on the context */
int ohg_context_launches(ohg_context* ctx, unsigned long long* out);
/* number of times the host has waited on the context's stream */
int ohg_context_syncs(ohg_context* ctx, unsigned long long* out);
/* number of device allocations the library has made on the context (no
 * counterpart in the reference: the reference allocates through Read<T>) */
int ohg_context_allocations(ohg_context* ctx, unsigned long long* out);
/* the context's cudaStream_t, for callers that order their own work on it */
int ohg_context_stream(ohg_context* ctx, void** stream_out);
/* Measurement hooks (no counterpart in the reference): when on, named hot
 * kernels ("coarsen_filter") record CUDA events around each launch on the
 * context's stream; ohg_context_kernel_time sums their durations and
 * algorithmic bytes since the last reset. */
int ohg_context_time_kernels(ohg_context* ctx, int on);
int ohg_context_kernel_time(ohg_context* ctx, const char* name, double* total_ms,
                            double* total_bytes, int* launches, int reset);
/* Precision mode of the cavity-quality and overshoot stages (no counterpart
 * in the reference, which computes in FP64 throughout).  on = 1 (default):
 * FP32 enclosures of the FP64 lengths and qualities decide wherever they
 * settle a comparison, and the rest is recomputed in FP64 with the
 * reference's arithmetic, so decisions and output reals equal FP64's.
 * on = 0: FP64 throughout. */
int ohg_context_set_screening(ohg_context* ctx, int on);
/* screening counters since the last reset: [0] cavity tets screened,
 * [1] tets recomputed in FP64, [2] edge lengths screened, [3] edge lengths
 * recomputed in FP64 */
int ohg_context_screen_counts(ohg_context* ctx, unsigned long long* counts4, int reset);

/* Launch-shape autotuner (no counterpart in the reference, whose launches
 * use Kokkos' fixed policies).  Tuned sites are the element-wise launches of
 * at least 65,536 items (block 128, 256 or 512 threads) and the persistent
 * coarsen screen (block 256 or 512, queue chunk 64 or 32), each per size
 * class (log2 of the item count).  Every variant computes the same results.
 * mode 0: defaults; 1: explore (each site's first launch runs the default
 * untimed, the next ones each variant once, timed by CUDA events read at the
 * next host wait; the site then keeps the fastest); 2 (default): frozen, the
 * choices made so far and the defaults elsewhere.  force >= 0 makes every
 * tuned site run variant (force mod its variant count); -1 ends that. */
int ohg_context_autotune(ohg_context* ctx, int mode);
int ohg_context_force_variant(ohg_context* ctx, int force);
/* tuned sites so far: [0] sites seen, [1] sites with a choice, [2] sites
 * whose choice is not the default variant */
int ohg_context_tuning(ohg_context* ctx, int* counts3);

/* ---- meshes ---- */
/* build_box on the unit square/cube with n subdivisions per axis, Hilbert
 * renumbered and classified (build_box, src/Omega_h_build.cpp:136-149) */
int ohg_build_box(ohg_context* ctx, int dim, int n, ohg_mesh** out);
/* seeded jitter of interior vertices (uniform +-0.15/n per axis) and an
 * analytic metric: 0 isotropic h=0.05+0.1|x0-0.5|, 1 shock, 2 boundary
 * layer, 3 isotropic sine, as packed tensors; 10 and 13: kinds 0 and 3 as
 * one scalar per vertex (an isotropic metric) */
int ohg_mesh_apply_workload(ohg_mesh* mesh, int n, unsigned long long seed, int metric_kind);
/* build_from_elems_and_coords (src/Omega_h_build.cpp:100-105): elements to
 * vertices plus coordinates and metric, all device arrays copied in */
int ohg_mesh_from_elems(ohg_context* ctx, int dim, int nverts, int nelems,
                        const int* ev2v_dev, const double* coords_dev,
                        const double* metric_dev, ohg_mesh** out);
/* A mesh from its stored arrays, as an Omega_h::Mesh holds them: for each
 * dimension d = 1..dim the downward adjacency d -> d-1 (down_dev[d], with
 * alignment codes codes_dev[d] for d >= 2), classification per dimension,
 * vertex coordinates and metric (Mesh::set_ents, src/Omega_h_mesh.cpp:87-95;
 * tags "class_dim", "class_id", "coordinates", "metric").  nents[d] entities
 * of each dimension; arrays are copied in, from device or host memory (the
 * kind is inferred from each address: pinned host memory is read by DMA),
 * and the call returns after the copies completed. */
int ohg_mesh_from_arrays(ohg_context* ctx, int dim, const int* nents,
                         const int* const* down_dev, const signed char* const* codes_dev,
                         const signed char* const* class_dim_dev,
                         const int* const* class_id_dev, const double* coords_dev,
                         const double* metric_dev, ohg_mesh** out);
/* a device copy of a mesh's stored arrays (derived adjacencies are not copied) */
int ohg_mesh_clone(ohg_mesh* mesh, ohg_mesh** out);
/* a copy of a mesh owned by another context (no counterpart in the
 * reference): the source context's stream is waited on, then the copies run
 * on the target context's stream */
int ohg_mesh_clone_to(ohg_mesh* src, ohg_context* ctx, ohg_mesh** out);
/* .osh files, the reference's binary mesh format, one part (binary::write
 * and binary::read, src/Omega_h_file.cpp:355-450 and :488-505): path is the
 * directory holding 0.osh, nparts and version.  The writer gives the bytes
 * the reference writes for the same mesh state: tags in the reference's
 * order, its partitioning flag, the box's class sets; compress = 1 writes
 * zlib streams (the system's libz, loaded at run time; ohg_osh_zlib tells
 * whether it was found).  The reader takes versions 1-9; tags other than
 * coordinates, metric, class_id, class_dim, global, length and quality are
 * kept as they are and written back, until an operator rebuilds the mesh.
 * Meshes of several parts, non-simplex families and parent links are
 * refused with OHG_ERR_INVALID. */
int ohg_mesh_write_osh(ohg_mesh* mesh, const char* path, int compress);
int ohg_mesh_read_osh(ohg_context* ctx, const char* path, ohg_mesh** out);
int ohg_osh_zlib(int* available);
int ohg_mesh_destroy(ohg_mesh* mesh);
int ohg_mesh_dim(ohg_mesh* mesh, int* out);
int ohg_mesh_nents(ohg_mesh* mesh, int dim, int* out);
/* Device memory held by a mesh: its arrays, derived adjacencies and caches,
 * each buffer once (no counterpart in the reference; the serving loop's
 * admission counts it). */
int ohg_mesh_device_bytes(ohg_mesh* mesh, long long* bytes);
/* The device's stream-ordered memory pool, which every context of the device
 * in this process draws from: bytes in use (including the freed blocks each
 * context keeps for reuse, up to 2 GiB per context), bytes reserved from
 * the device, and the high-water mark of bytes in use (reset to the current
 * use when reset_high is nonzero).  It neither waits on nor touches the context's
 * stream, so any host thread may call it.  No counterpart in the reference. */
int ohg_context_pool_bytes(ohg_context* ctx, int reset_high, long long* used,
                           long long* reserved, long long* used_high);
/* Size in bytes of a named mesh array, then a copy of it into caller device
 * memory.  Names: coords, metric, length, quality, ev2v_<d>, down_<d>,
 * downcodes_<d>, class_dim_<d>, class_id_<d>, global_<d>, up_a2ab_<lo><hi>,
 * up_ab2b_<lo><hi>, up_codes_<lo><hi>, down31, downcodes31,
 * star_a2ab_<d>, star_ab2b_<d>, dual_a2ab, dual_ab2b (Mesh::ask_adj,
 * src/Omega_h_mesh.cpp:347-357; tags, src/Omega_h_mesh.hpp:62-78) */
int ohg_mesh_array_bytes(ohg_mesh* mesh, const char* name, long long* nbytes);
/* copies a named array to dst, device memory or host memory (pinned host
 * memory is copied to by DMA); returns after the copy completed */
int ohg_mesh_get_array(ohg_mesh* mesh, const char* name, void* dst, long long capacity_bytes);
/* ohg_mesh_get_array for n arrays at once: names[i] into dsts[i] (capacity
 * caps[i] bytes), all copies queued before one wait.  Every name and
 * capacity is checked before any copy starts. */
int ohg_mesh_get_arrays(ohg_mesh* mesh, int n, const char* const* names, void* const* dsts,
                        const long long* caps);
/* replaces vertex coordinates or metric ("coords" | "metric").  A metric of
 * nverts values is isotropic (the reference's one-component metric tag: its
 * scalar lengths, sizes, maxdet and log-Euclidean means are used), one of
 * nverts * 6 (3D) or * 3 (2D) values is a packed tensor.  src may be device
 * or host memory; the call returns after the copy completed. */
int ohg_mesh_set_array(ohg_mesh* mesh, const char* name, const void* src_dev, long long nbytes);

/* ---- the pass ---- */
/* AdaptOpts::AdaptOpts(Int dim) defaults (src/Omega_h_adapt.cpp:52-85) */
int ohg_adapt_opts_default(int dim, ohg_adapt_opts* out);
/* refine_by_size -> coarsen_by_size -> swap_edges when the minimum element
 * quality is below min_quality_desired (src/Omega_h_adapt.cpp:173-210) */
int ohg_adapt_pass(ohg_mesh* mesh, const ohg_adapt_opts* opts, ohg_pass_stats* stats);
/* Omega_h::adapt (src/Omega_h_adapt.cpp:272-288) for meshes without
 * conservation tags or geometry: refine/coarsen by size until lengths
 * settle, then edge swaps and sliver collapses (coarsen_slivers,
 * src/Omega_h_coarsen.cpp:210-220) until the worst quality reaches
 * min_quality_desired or nothing helps */
int ohg_adapt(ohg_mesh* mesh, const ohg_adapt_opts* opts, ohg_adapt_result* result);
/* coarsen_slivers (src/Omega_h_coarsen.cpp:210-220) */
int ohg_coarsen_slivers(ohg_mesh* mesh, const ohg_adapt_opts* opts, int* did);
/* ---- batches of meshes (no counterpart in the reference) ----
 * The disjoint union of n meshes of one dimension is one mesh; one adapt
 * pass over it gives, mesh by mesh, bit for bit the result of n separate
 * passes (every decision is local to a mesh and numbering order within a
 * mesh is kept), in the launches of a single pass.  Class ids must lie in
 * [0, 2^20) and n <= 2047. */
int ohg_mesh_concat(ohg_context* ctx, ohg_mesh* const* meshes, int n, ohg_mesh** union_out);
/* the n parts of a union after any number of passes, as new mesh handles
 * sharing the union's device memory; the union handle is consumed in the
 * sense that its arrays are rewritten (destroy it after splitting) */
int ohg_mesh_split(ohg_mesh* union_mesh, int n, ohg_mesh** parts_out);
/* concat, one adapt pass, split: each meshes[i] is replaced by its result;
 * stats are those of the union pass */
int ohg_adapt_pass_batch(ohg_context* ctx, ohg_mesh* const* meshes, int n,
                         const ohg_adapt_opts* opts, ohg_pass_stats* stats);
/* one operator each; *did = whether the mesh changed
 * (src/Omega_h_refine.hpp:8, src/Omega_h_coarsen.hpp:44, src/Omega_h_swap.hpp:14) */
int ohg_refine_by_size(ohg_mesh* mesh, const ohg_adapt_opts* opts, int* did);
int ohg_coarsen_by_size(ohg_mesh* mesh, const ohg_adapt_opts* opts, int* did);
int ohg_swap_edges(ohg_mesh* mesh, const ohg_adapt_opts* opts, int* did);

/* ---- stage kernels on a mesh ---- */
/* measure_edges_metric (src/Omega_h_shape.cpp:28-44); a2e_dev NULL = all */
int ohg_measure_edges_metric(ohg_mesh* mesh, const int* a2e_dev, int n, double* out_dev);
/* measure_qualities (src/Omega_h_quality.cpp:25-44); a2e_dev NULL = all */
int ohg_measure_qualities(ohg_mesh* mesh, const int* a2e_dev, int n, double* out_dev);
/* FP32 enclosures [lo, hi] of the FP64 quality (src/Omega_h_quality.hpp:8-52)
 * of n simplices given as vertex (dim+1)-tuples of the mesh, with the FP64
 * value itself; the screening step of the precision mode, exposed for
 * checking it (no counterpart in the reference) */
int ohg_screen_tet_qualities(ohg_mesh* mesh, const int* tv2v_dev, int n, float* lo_dev,
                             float* hi_dev, double* exact_dev);
/* the same intervals by the collapse screen's per-face route: the face
 * opposite vertex slot `slot` (0..3) of each tet taken as fixed, its
 * invariants made once, and the vertex at `slot` as the one moved onto;
 * cubed != 0: [lo, hi] bounds the cube of the quality, as the 3D collapse
 * screen compares it (a 3D mesh only; exposed for checking it) */
int ohg_screen_tet_qualities_face(ohg_mesh* mesh, const int* tv2v_dev, int n, int slot,
                                  int cubed, float* lo_dev, float* hi_dev, double* exact_dev);
/* the same for the metric length (edge_length, src/Omega_h_shape.hpp:112-157)
 * of n vertex pairs */
int ohg_screen_edge_lengths(ohg_mesh* mesh, const int* ev2v_dev, int n, float* lo_dev,
                            float* hi_dev, double* exact_dev);
/* get_mident_metrics for edges (src/Omega_h_metric.cpp:73-101): 6 per edge */
int ohg_get_mident_metrics(ohg_mesh* mesh, const int* edges_dev, int n, double* out_dev);
/* refine_qualities (src/Omega_h_refine_qualities.cpp:88-107) */
int ohg_refine_qualities(ohg_mesh* mesh, const int* cands2edges_dev, int n, double* out_dev);
/* check_collapse_class / check_collapse_exposure (src/Omega_h_collapse.hpp:30-33) */
int ohg_check_collapse_class(ohg_mesh* mesh, const int* cands2edges_dev, int n,
                             const signed char* codes_dev, signed char* out_dev);
int ohg_check_collapse_exposure(ohg_mesh* mesh, const int* cands2edges_dev, int n,
                                const signed char* codes_dev, signed char* out_dev);
/* prevent_coarsen_overshoot (src/Omega_h_coarsen.hpp:20-21) */
int ohg_prevent_coarsen_overshoot(ohg_mesh* mesh, double max_length, const int* cands2edges_dev,
                                  int n, const signed char* codes_dev, signed char* out_dev);
/* coarsen_qualities (src/Omega_h_coarsen.hpp:15): 2 per candidate, -1 where
 * that direction does not collapse */
int ohg_coarsen_qualities(ohg_mesh* mesh, const int* cands2edges_dev, int n,
                          const signed char* codes_dev, double* out2_dev);
/* choose_rails (src/Omega_h_coarsen.hpp:24-26): per-vertex outputs */
int ohg_choose_rails(ohg_mesh* mesh, const int* cands2edges_dev, int n,
                     const signed char* codes_dev, const double* quals2_dev,
                     signed char* vert_cands_dev, double* vert_quals_dev,
                     long long* vert_rails_dev);
/* mark_sliver_layers (src/Omega_h_mark.hpp:23) */
int ohg_mark_sliver_layers(ohg_mesh* mesh, double qual_ceil, int nlayers, signed char* out_dev);
/* swap2d_qualities (src/Omega_h_swap2d_qualities.cpp:70-81): 2D meshes */
int ohg_swap2d_qualities(ohg_mesh* mesh, double max_length_allowed, const int* cands2edges_dev,
                         int n, double* quals_dev);
/* swap3d_qualities (src/Omega_h_swap3d.hpp:9-10) */
int ohg_swap3d_qualities(ohg_mesh* mesh, double max_length_allowed, const int* cands2edges_dev,
                         int n, double* quals_dev, signed char* configs_dev);
/* swap3d::find_loop (src/Omega_h_swap3d_loop.hpp:24-78) for n edges: the
 * number of tets around each edge (0 when outside 3..7), the edge's two
 * vertices (2 ints per edge) and the loop vertices ordered to curl around
 * it (7 ints per edge, unused slots 0); device arrays */
int ohg_swap3d_find_loops(ohg_mesh* mesh, const int* edges_dev, int n, int* sizes_dev,
                          int* eev2v_dev, int* loop_verts_dev);
/* find_indset over the mesh's star graph (src/Omega_h_indset.hpp:11-14) */
int ohg_find_indset(ohg_mesh* mesh, int ent_dim, const double* quality_dev,
                    const signed char* candidates_dev, signed char* out_dev, int* rounds);

/* Times one stage kernel alone on this mesh: "lengths" (all edges),
 * "qualities" (all elements), "refine_qualities" (every edge a candidate),
 * "coarsen_qualities" (every edge, both directions).  Each of reps launches
 * is bracketed by CUDA events on the context stream after a 256 MiB write
 * that evicts L2; *avg_ms is the mean launch time and *alg_bytes the
 * compulsory bytes of one launch (each input array read once, each output
 * written once).  A measurement hook with no counterpart in the reference. */
int ohg_time_stage(ohg_mesh* mesh, const char* stage, int reps, float* avg_ms, double* alg_bytes);
/* Measurement hook (no counterpart in the reference): the device's FP64
 * fused multiply-add throughput in GFLOP/s, from chains of dependent FMAs
 * timed with CUDA events on the context's stream (best of reps launches). */
int ohg_fp64_peak(ohg_context* ctx, int reps, double* gflops);

/* ---- graph-level kernels (no mesh) ---- */
/* invert_adj (src/Omega_h_adj.cpp:231-263): outputs nlows+1, nhigh*k, nhigh*k */
int ohg_invert_adj(ohg_context* ctx, const int* hl2l_dev, const signed char* codes_dev,
                   int nhigh, int nlows_per_high, int nlows, int* a2ab_dev, int* ab2b_dev,
                   signed char* codes_out_dev);
/* reflect_down (src/Omega_h_adj.cpp:424-441) given the low entities' vertices
 * and the vertex-to-low upward adjacency; outputs nhigh*nlows_per_high */
int ohg_reflect_down(ohg_context* ctx, const int* hv2v_dev, int nhigh, int high_dim,
                     int low_dim, const int* lv2v_dev, int nlows, const int* v2l_a2ab_dev,
                     const int* v2l_ab2b_dev, const signed char* v2l_codes_dev, int nverts,
                     int* hl2l_dev, signed char* codes_out_dev);
/* find_indset on an explicit graph (src/Omega_h_indset.cpp:17-34), entity
 * numbers as global numbers.  *rounds: the rounds run; the rounds update
 * their states in place, so the count (never the set) depends on the launch
 * schedule */
int ohg_find_indset_graph(ohg_context* ctx, int n, const int* xadj_dev, const int* adj_dev,
                          const double* quality_dev, const signed char* candidates_dev,
                          signed char* out_dev, int* rounds);
/* sort_by_keys (src/Omega_h_sort.cpp:71-92): stable lexicographic sort of n
 * tuples of width int32 (key_bytes 4) or int64 (key_bytes 8) keys */
int ohg_sort_by_keys(ohg_context* ctx, const void* keys_dev, int n, int width, int key_bytes,
                     int* perm_dev);
/* hilbert::sort_coords (src/Omega_h_hilbert.cpp:52-55) */
int ohg_hilbert_sort(ohg_context* ctx, const double* coords_dev, int n, int dim, int* perm_dev);
/* hilbert::AxestoTranspose then hilbert::untranspose
 * (src/Omega_h_hilbert.hpp:65-117), Skilling's transform, for n points of
 * dim (1..3) integer coordinates of bits (1..64) bits each: the Hilbert
 * index as dim words of bits bits, most significant word first; device
 * arrays of dim words per point.  A coordinate of more than bits bits sets
 * OHG_ERR_BOUNDS. */
int ohg_hilbert_transpose(ohg_context* ctx, const unsigned long long* axes_dev, int n, int dim,
                          int bits, unsigned long long* keys_dev);
/* offset_scan (src/Omega_h_int_scan.cpp:10-20): n+1 outputs */
int ohg_offset_scan(ohg_context* ctx, const int* counts_dev, int n, int* out_dev);
/* collect_marked (src/Omega_h_map.cpp:174-185): the indices i < n with
 * marks_dev[i] != 0, in increasing order, into out_dev (room for n ints);
 * their number into *count (host) */
int ohg_collect_marked(ohg_context* ctx, const signed char* marks_dev, int n, int* out_dev,
                       int* count);
/* Self-test of failure detection, no counterpart in the reference: runs the
 * single-pass scan of n counts (n > 4096, device memory) with its first tile
 * withheld, so the other tiles' bounded waits on it run out (under a second).
 * Returns OHG_ERR_TIMEOUT when the limit works; the context stays usable.
 * out_dev (n+1 ints) is scratch. */
int ohg_selftest_scan_wait_limit(ohg_context* ctx, const int* counts_dev, int n, int* out_dev);
/* offset_scan without any device allocation: no counterpart in the
 * reference.  For hosts that cannot let the library allocate at that moment
 * (their own arena owns the device memory, or they are recovering from an
 * out-of-memory failure and need offsets to compact before freeing).  The
 * scan's tile sums live in one fixed device array per device, sized for at
 * most ohg_offset_scan_noalloc_limit() counts (4,194,304); larger n fails
 * with OHG_ERR_INVALID before any launch.  The first call on a device looks
 * up the array's address; make that first call before any stream capture.
 * Like every entry point here, the call waits for the context's stream
 * before it returns (it reads the status word).  Nothing has to be zeroed
 * beforehand.  Calls in flight on one device at the
 * same time (other streams, contexts or threads) race on the shared array:
 * order them. */
int ohg_offset_scan_noalloc(ohg_context* ctx, const int* counts_dev, int n, int* out_dev);
int ohg_offset_scan_noalloc_limit(int* max_counts);

/* ---- metric tools (src/Omega_h_metric.cpp, src/Omega_h_metric_input.cpp)
 * Metrics are packed symmetric tensors per vertex: (xx, yy, zz, yx, zy, zx)
 * in 3D, (xx, yy, yx) in 2D; all pointers are device pointers.  Every
 * function computes in FP64 with the reference's operation order.  A
 * failed eigendecomposition sets the device status, returned as
 * OHG_ERR_NUMERIC. */
/* find_polynomial_roots (src/Omega_h_eigen.hpp:21-85) of n monic cubics
 * x^3 + a_2 x^2 + a_1 x + a_0, coefficients (a_0, a_1, a_2) per cubic:
 * the number of distinct roots, 3 roots and 3 multiplicities per cubic;
 * roots closer than eps are merged (the reference's default is 1e-6, its
 * eigensolver uses 5e-5) */
int ohg_cubic_roots(ohg_context* ctx, int n, const double* coeffs_dev, double eps,
                    int* nroots_dev, double* roots_dev, int* mults_dev);
/* decompose_eigen (src/Omega_h_eigen.hpp:278-293) of n dim x dim matrices
 * (dim 2 or 3) stored by columns: q (by columns) holds the eigenvectors, l
 * the eigenvalues; a failed decomposition returns OHG_ERR_NUMERIC */
int ohg_decompose_eigen(ohg_context* ctx, int dim, int n, const double* m_dev, double* q_dev,
                        double* l_dev);
/* intersect_metrics (src/Omega_h_metric.cpp:536-557), including Barral's
 * degenerate cases where eigenvalues are below 1e-10
 * (src/Omega_h_metric_intersect.hpp:25-212) */
int ohg_intersect_metrics(ohg_context* ctx, int dim, int n, const double* a, const double* b,
                          double* out);
/* clamp_metrics (src/Omega_h_metric.cpp:36-56): eigenvalues into
 * [1/h_max^2, 1/h_min^2] */
int ohg_clamp_metrics(ohg_context* ctx, int dim, int n, const double* metrics, double h_min,
                      double h_max, double* out);
/* get_hessian_metrics (src/Omega_h_metric.cpp:332-368) */
int ohg_hessian_metrics(ohg_context* ctx, int dim, int n, const double* hessians, double eps,
                        double* out);
/* get_implied_metrics (src/Omega_h_metric.cpp:304-309): out holds nverts
 * metrics */
int ohg_mesh_implied_metrics(ohg_mesh* mesh, double* out);
/* limit_metric_gradation (src/Omega_h_metric.cpp:199-220); steps (may be
 * null) receives the number of sweeps */
int ohg_mesh_limit_metric_gradation(ohg_mesh* mesh, const double* metrics, double max_rate,
                                    double tol, double* out, int* steps);
/* get_expected_nelems (src/Omega_h_metric.cpp:516-519), summed exactly */
int ohg_mesh_expected_nelems(ohg_mesh* mesh, const double* metrics, double* out);

/* MetricSource / MetricInput (src/Omega_h_metric_input.cpp:13-35).  type:
 * 0 constant (knob = length), 3 given (the metrics in `given`, scaled by
 * 1/knob^2), 4 implied (scaled by 1/knob^2); variation (1), derivative (2)
 * and curvature (5) are refused.  isotropy: 0 anisotropic, 2 iso-size
 * (1, iso-length, is refused).  scales: 0 absolute, 1 scaled by the
 * element-count iteration.  At least one source must stay anisotropic. */
typedef struct ohg_metric_source {
  int type;
  double knob;
  int isotropy;
  int scales;
  const double* given;
} ohg_metric_source;
typedef struct ohg_metric_input {
  int nsources;
  ohg_metric_source sources[8];
  int should_limit_lengths;
  double min_length, max_length;
  int should_limit_gradation;
  double max_gradation_rate, gradation_convergence_tolerance;
  int should_limit_element_count;
  double max_element_count, min_element_count, element_count_over_relaxation;
  int nsmoothing_steps;
} ohg_metric_input;
/* MetricInput() defaults (src/Omega_h_metric_input.cpp:23-35), no sources */
int ohg_metric_input_default(ohg_metric_input* out);
/* generate_metrics (src/Omega_h_metric_input.cpp:140-275): out holds
 * nverts metrics; niters (may be null) the element-count iterations */
int ohg_mesh_generate_metrics(ohg_mesh* mesh, const ohg_metric_input* in, double* out,
                              int* niters);

#ifdef __cplusplus
}
#endif
#endif
