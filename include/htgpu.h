/*
 * htgpu.h -- C ABI of libhtgpu, the GB300 (sm_103a) implementation of htool's
 * H-matrix hot path: cluster/block trees, device partialACA assembly and the
 * H-matrix product over all leaves.
 *
 * Every function returns HTGPU_OK (0) or an error code; htgpu_last_error()
 * gives the message of the calling thread's last failure (messages keep
 * htool's "[Htool error] ..." prefix).  No C++ exception crosses this
 * boundary.  Handles are not thread-safe: one thread per handle at a time,
 * like htool's HMatrix, whose products mutate its `infos` map
 * (include/htool/types/hmatrix.hpp:87).
 *
 * Each declaration names the upstream htool 0.8.1 interface it replaces
 * (paths relative to the htool source tree).
 */
#ifndef HTGPU_H
#define HTGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define HTGPU_OK 0
#define HTGPU_ERR_INVALID 1     /* invalid argument (std::invalid_argument upstream) */
#define HTGPU_ERR_UNSUPPORTED 2 /* valid htool input this library does not handle */
#define HTGPU_ERR_CUDA 3        /* CUDA runtime error */
#define HTGPU_ERR_NOMEM 4       /* host allocation failure */
#define HTGPU_ERR_INTERNAL 5    /* inconsistent device result (a bug) */

/* flags of the product entry points */
#define HTGPU_HOST_PTRS 1u         /* in/out are host memory; the call is synchronous */
#define HTGPU_CLUSTER_NUMBERING 2u /* in/out are in cluster (permuted) order: no permutation */
#define HTGPU_GLOBAL_TO_LOCAL 4u   /* in: the whole input in cluster order; out: the local rows of the handle's MPI rank */

/* built-in device generators (the device-generator variant of
 * VirtualGenerator<T>::copy_submatrix, include/htool/types/virtual_generator.hpp:22) */
#define HTGPU_KERNEL_INV_R_EPS 0 /* 1 / (1e-5 + |x - y|) */
#define HTGPU_KERNEL_LAPLACE 1   /* 1 / (4 pi |x - y|), 0 where x == y */
#define HTGPU_KERNEL_HELMHOLTZ 2 /* exp(i k |x - y|) / (4 pi |x - y|), 0 where x == y; complex handles only */

typedef struct htgpu_cluster_s *htgpu_cluster;
typedef struct htgpu_hmatrix_s *htgpu_hmatrix;
typedef struct htgpu_mlp_s *htgpu_mlp;
typedef struct htgpu_batch_s *htgpu_batch;

/* Message of the calling thread's last failed call ("" if none). */
const char *htgpu_last_error(void);

/* Library version (htool_gb300 major.minor). */
int htgpu_version(int *major, int *minor);

/* ---------------------------------------------------------------------------
 * Cluster trees
 * -------------------------------------------------------------------------*/

/* Replaces Cluster<PCA<SplittingTypes::GeometricSplitting>>::build(nb_pt, x, nb_sons)
 * (include/htool/clustering/cluster.hpp:94-97, 57-92; pca.hpp:15-128) after
 * set_minclustersize (cluster.hpp:334), on one MPI rank.  xyz: n points, xyz
 * interleaved.  nb_sons: 2 or -1 (automatic = 2).  The tree, permutation,
 * centres and radii are bit-identical to htool's. */
int htgpu_cluster_build(int n, const double *xyz, int minclustersize, int nb_sons, htgpu_cluster *out);
int htgpu_cluster_destroy(htgpu_cluster c);

/* The same build as rank `rank` of a run of size_world MPI ranks would do it
 * (cluster.hpp:57-92 with MPI_Comm_size = size_world): the root is split
 * into one son per rank (pca.hpp:28), son p holding rank p's points
 * (pca.hpp:93-99).  The tree does not depend on the rank, which only picks
 * the local cluster; htgpu_hmatrix_set_local_rank gives it to an H-matrix.
 * size_world = 1 is htgpu_cluster_build. */
int htgpu_cluster_build_world(int n, const double *xyz, int minclustersize, int nb_sons, int size_world, htgpu_cluster *out);

/* A forest (no counterpart in the reference): k independent cluster trees
 * side by side, their points concatenated in order (member q's points are
 * offsets[q] .. offsets[q + 1]).  An H-matrix on forests holds the
 * block-diagonal union of the members' H-matrices: each member's block tree
 * is htool's on its own pair of trees (no block couples two members), so a
 * build, a product or a batch launch handles every member at once.  Inputs
 * and outputs are the members' vectors concatenated (user numbering of each
 * member shifted by its offset).  Members must be one-rank trees. */
int htgpu_cluster_forest(int k, const htgpu_cluster *members, htgpu_cluster *out);
/* *k and, when offsets != NULL, the k + 1 member offsets of a forest (k = 0
 * for an ordinary tree). */
int htgpu_cluster_forest_offsets(htgpu_cluster c, int *k, int *offsets);

/* get_masteroffset (cluster.hpp:42, virtual_cluster.hpp:61-62):
 * *size_world, and when mo != NULL, mo[2 p] = offset and mo[2 p + 1] =
 * size of rank p's cluster (cluster numbering). */
int htgpu_cluster_masteroffset(htgpu_cluster c, int *size_world, int *mo);

/* A cluster tree built elsewhere, e.g. any htool VirtualCluster
 * (include/htool/clustering/virtual_cluster.hpp:28-40) walked in pre-order:
 * perm[n] (get_perm) and per node, sons in order, node_i[6 * k ...] =
 * depth, rank, offset, size, nb_sons, counter and node_d[4 * k ...] = rad,
 * ctr[0..2] (the layout of htgpu_cluster_get_nodes).  The sons of every
 * node must tile its points. */
int htgpu_cluster_import(int n, const int *perm, int nnodes, const int *node_i, const double *node_d, htgpu_cluster *out);

/* Sizes: number of points, number of nodes, get_min_depth/get_max_depth
 * (cluster.hpp:277-278). */
int htgpu_cluster_info(htgpu_cluster c, int *n, int *nnodes, int *min_depth, int *max_depth);

/* get_perm (cluster.hpp:279): perm[n]. */
int htgpu_cluster_get_perm(htgpu_cluster c, int *perm);

/* Every node in pre-order (sons in order): node_i[6 * k ...] = depth, rank,
 * offset, size, nb_sons, counter; node_d[4 * k ...] = rad, ctr[0..2]
 * (VirtualCluster getters, include/htool/clustering/virtual_cluster.hpp:28-40). */
int htgpu_cluster_get_nodes(htgpu_cluster c, int *node_i, double *node_d);

/* Block::build(UPLO = 'N') local task list (include/htool/blocks/blocks.hpp:237-278):
 * call with out = NULL to get *ntasks, then with room for 5 * ntasks ints:
 * t.offset, t.size, s.offset, s.size, admissible. */
int htgpu_block_tasks(htgpu_cluster t, htgpu_cluster s, double eta, int *ntasks, int *out);

/* The same for Block::build(UPLO, force_sym) (blocks.hpp:237-278): uplo 'U' /
 * 'L' keeps the tasks of one triangle (s.offset >= t.offset / <=); with
 * uplo != 'N' or force_sym the tree is build_sym_block_tree's
 * (blocks.hpp:140-235). */
int htgpu_block_tasks_sym(htgpu_cluster t, htgpu_cluster s, double eta, char uplo, int force_sym, int *ntasks, int *out);

/* Block::build(UPLO = 'N') local task list of MPI rank `rank` of the run
 * the trees were built for (blocks.hpp:251-277: tasks whose target cluster
 * belongs to that rank, sorted by offsets). */
int htgpu_block_tasks_rank(htgpu_cluster t, htgpu_cluster s, double eta, int rank, int *ntasks, int *out);

/* ---------------------------------------------------------------------------
 * H-matrices (double precision, non-symmetric storage)
 * -------------------------------------------------------------------------*/

/* Replaces HMatrix<double>(cluster_tree_t, cluster_tree_s, epsilon, eta, 'N', 'N')
 * (include/htool/types/hmatrix.hpp:115-122) followed by
 * set_compression(std::make_shared<partialACA<double>>()) (hmatrix.hpp:220).
 * The matrix lives on CUDA device `device`. */
int htgpu_hmatrix_create(htgpu_cluster t, htgpu_cluster s, double epsilon, double eta, int device, htgpu_hmatrix *out);
int htgpu_hmatrix_destroy(htgpu_hmatrix h);

/* HMatrix<std::complex<double>>(t, s, epsilon, eta) (hmatrix.hpp:44-270)
 * with partialACA; build with HTGPU_KERNEL_HELMHOLTZ (exp(i k r)/(4 pi r),
 * 0 at r = 0, k = kernel_param).  Complex vectors are interleaved (re, im)
 * doubles, column-major per right-hand side (std::complex<double> layout):
 * every product entry point takes them with twice the real sizes.  The
 * matrix is stored and applied in real form (entry z -> [[re, -im],
 * [im, re]]), so every storage policy and the batched products apply;
 * htgpu_hmatrix_get_leaves / get_factors describe that real form;
 * htgpu_hmatrix_mvprod_transp gives the plain transpose (htool's op 'T'). */
int htgpu_hmatrix_create_complex(htgpu_cluster t, htgpu_cluster s, double epsilon, double eta, int device, htgpu_hmatrix *out);

/* The storage of a complex handle, chosen before its build: 0 (default) the
 * real form above; 1 the native complex layout, at half the factor and
 * dense bytes of the real form (htool's own std::complex<double> storage:
 * U, V and dense blocks at 16 bytes an entry, lrmat/lrmat.hpp:89-100): a
 * leaf U V is stored as Re U, Im U and one tile holding the (Re, Im) pairs
 * of V's entries, a dense block as the (Re, Im) pairs of its entries; a
 * product runs the real kernels with twice the right-hand sides (the input
 * as x and i x, the tiles' sums a followed by i a).  The native layout takes
 * symmetry 'N' and partialACA, FP64 or reduced precision (one column
 * scale for the Re U and Im U columns of a complex column), and every
 * product but the allocation-free one (htgpu_hmatrix_mvprod in any
 * numbering, htgpu_hmatrix_mvprod_global_to_local,
 * htgpu_hmatrix_mvprod_transp: the plain transpose from a twin in the same
 * layout, batches, autotune); the digit planes, symmetric handles and the
 * allocation-free product return HTGPU_ERR_UNSUPPORTED; dumps record the
 * layout and reload into a handle of the same layout.
 * htgpu_hmatrix_set_leaves / get_leaves / get_factors take and give
 * htool's complex leaves (sizes of the points, entries as interleaved
 * (re, im) doubles). */
int htgpu_hmatrix_set_complex_layout(htgpu_hmatrix h, int native);
int htgpu_hmatrix_get_complex_layout(htgpu_hmatrix h, int *native);

/* set_maxblocksize / set_mintargetdepth / set_minsourcedepth (hmatrix.hpp:213-215). */
int htgpu_hmatrix_set_maxblocksize(htgpu_hmatrix h, unsigned int maxblocksize);
int htgpu_hmatrix_set_mintargetdepth(htgpu_hmatrix h, unsigned int depth);
int htgpu_hmatrix_set_minsourcedepth(htgpu_hmatrix h, unsigned int depth);

/* Replaces HMatrix<double>::build(mat, xt, xs) (hmatrix.hpp:286-341) where
 * mat is a built-in device generator (HTGPU_KERNEL_*) evaluated on the GPU;
 * every admissible block is compressed by device partialACA
 * (include/htool/lrmat/partialACA.hpp:39-171), batched across blocks, with
 * htool's rejection and recursion rules (hmatrix.hpp:504-607).  xt / xs are
 * the host point arrays used to build the cluster trees. */
int htgpu_hmatrix_build(htgpu_hmatrix h, int kernel_id, double kernel_param, const double *xt, const double *xs);

/* HMatrix<double>::build(mat, xt) (hmatrix.hpp:343-400): one point array
 * for rows and columns and the symmetric block tree (force_sym). */
int htgpu_hmatrix_build_sym(htgpu_hmatrix h, int kernel_id, double kernel_param, const double *xt);

/* A host generator: VirtualGenerator<double>::copy_submatrix(M, N, rows,
 * cols, ptr) (include/htool/types/virtual_generator.hpp:22) as a C callback:
 * fill ptr[i + M * j] = A(rows[i], cols[j]) (user numbering, ptr column-major
 * and owned by the library) and return 0, or nonzero to abort the build
 * (the call then fails with HTGPU_ERR_INVALID).  As in htool, where
 * HMatrix::build calls it from OpenMP threads (hmatrix.hpp:424-452), it is
 * called concurrently from several host threads and must be thread-safe. */
typedef int (*htgpu_generator_fn)(void *ctx, int M, int N, const int *rows, const int *cols, double *ptr);

/* Replaces HMatrix<double>::build(mat, xt, xs) (hmatrix.hpp:286-341) for a
 * user generator that lives on the host.  partialACA (lrmat/partialACA.hpp:
 * 39-171) runs on the device for every admissible block at once, one cross
 * per step: the library asks the generator for the residual row A(I, :) of
 * every unfinished block, then for the column A(:, J), in batches; dense
 * leaves are filled by one call each.  htool's rejection and recursion rules
 * and the current compression (set_compression) apply; with a generator
 * that returns the same entries the result equals htgpu_hmatrix_build's
 * (leaves, ranks and factors).  Real H-matrices only. */
int htgpu_hmatrix_build_host(htgpu_hmatrix h, htgpu_generator_fn gen, void *ctx, const double *xt, const double *xs);
/* HMatrix<double>::build(mat, xt) (hmatrix.hpp:343-400) with a host generator. */
int htgpu_hmatrix_build_host_sym(htgpu_hmatrix h, htgpu_generator_fn gen, void *ctx, const double *xt);

/* partialACA of one block with a host generator, on the device: the
 * counterpart of VirtualLowRankGenerator<double>::copy_low_rank_approximation
 * (include/htool/lrmat/virtual_lrmat_generator.hpp:15) as partialACA
 * implements it (lrmat/partialACA.hpp:39-171).  rows / cols: the block's
 * M and N user indices; xt (points, 3 doubles each, indexed by rows) and ctr
 * (the target cluster's centre) choose the first row as htool does (row 0
 * when either is NULL); reqrank: htool's rank argument (-1 adaptive to
 * epsilon, > 0 a required rank).  *rank: the rank, or -1 when the block is
 * not worth compressing (q (M + N) > M N), as htool returns it.  One handle
 * per host thread: a handle is not thread-safe. */
typedef struct htgpu_aca_s *htgpu_aca;
int htgpu_aca_create(int device, htgpu_aca *out);
int htgpu_aca_destroy(htgpu_aca a);
int htgpu_aca_compress(htgpu_aca a, htgpu_generator_fn gen, void *ctx, double epsilon, int M, int N, const int *rows, const int *cols, const double *xt, const double *ctr, int reqrank, int *rank);
/* The last compression's factors in htool's layouts (lrmat.hpp:47-50): U
 * (M x rank) and V (rank x N), column-major, into caller memory. */
int htgpu_aca_factors(htgpu_aca a, double *U, double *V);

/* Before a build: the symmetry and UPLO arguments of HMatrix's constructor
 * (hmatrix.hpp:115-122): 'N' with 'N', or 'S' / 'H' with 'U' / 'L' -- one
 * triangle of the block tree is stored (ComputeAdmissibleBlocksSym
 * recursion, hmatrix.hpp:610-700) and products apply every stored
 * off-diagonal leaf and its transpose ('S') or conjugate transpose ('H'),
 * diagonal blocks as symv / hemv read their UPLO triangle
 * (hmatrix.hpp:844-911, matrix.hpp:386-447); t and s must be the same tree.
 * 'H' needs a complex handle. */
int htgpu_hmatrix_set_symmetry(htgpu_hmatrix h, char symmetry, char uplo);
int htgpu_hmatrix_get_symmetry(htgpu_hmatrix h, char *symmetry, char *uplo);

/* Before a build: set_compression (hmatrix.hpp:220) with
 * HTGPU_COMPRESSION_PARTIAL_ACA (lrmat/partialACA.hpp:39-171, the default of
 * this library) or HTGPU_COMPRESSION_SYM_PARTIAL_ACA (lrmat/sympartialACA.hpp:
 * 28-210, htool's default: a block whose target comes before its source is
 * compressed as its mirror); real H-matrices only. */
#define HTGPU_COMPRESSION_PARTIAL_ACA 0
#define HTGPU_COMPRESSION_SYM_PARTIAL_ACA 1
int htgpu_hmatrix_set_compression(htgpu_hmatrix h, int compressor);

/* Adopt leaves built elsewhere, e.g. exported from an htool HMatrix through
 * get_MyFarFieldMats / get_MyNearFieldMats (hmatrix.hpp:193-198) and
 * LowRankMatrix::get_U / get_V (include/htool/lrmat/lrmat.hpp:65-66).
 * lr_desc[5 * b ...] = offset_i, offset_j, m, n, rank (cluster numbering);
 * uv = for each low-rank leaf in order, U (m x rank, column-major) then
 * V (rank x n, column-major); d_desc[4 * b ...] = offset_i, offset_j, m, n;
 * dense = each dense leaf m x n column-major.  Host memory; copied.  On a
 * handle with symmetry 'S' / 'H' the leaves are one triangle (diagonal
 * blocks dense and square, no block together with its mirror) and the
 * product adds every off-diagonal leaf's (conjugate) transpose.  A complex
 * handle in real form takes the leaves of the real form (every offset, size
 * and rank doubled, entries z as [[re, -im], [im, re]]); one in the native
 * complex layout takes htool's complex leaves as they are (sizes of the
 * points, uv and dense as interleaved (re, im) doubles). */
int htgpu_hmatrix_set_leaves(htgpu_hmatrix h, int nlr, const int *lr_desc, const double *uv, int ndense, const int *d_desc, const double *dense);

/* Replaces HMatrix<double>::mvprod_global_to_global(in, out, mu)
 * (hmatrix.hpp:1074-1182): out = H in for mu right-hand sides stored
 * column-major (in: nb_cols x mu, out: nb_rows x mu), in user numbering
 * unless HTGPU_CLUSTER_NUMBERING.  With HTGPU_HOST_PTRS the pointers are host
 * memory and the call returns when out is written; otherwise they are device
 * pointers and the call is ordered on `stream` (a cudaStream_t; NULL = the
 * handle's own stream; cudaStreamLegacy / cudaStreamPerThread select the
 * default streams) and returns at once. */
int htgpu_hmatrix_mvprod(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, void *stream);

/* The H-matrix of rank `rank` of a multi-rank run: on trees from
 * htgpu_cluster_build_world, the build keeps that rank's local tasks only
 * (htool's HMatrix::build on rank `rank`, hmatrix.hpp:286-341 with
 * blocks.hpp:258-273).  Call before the build; symmetry 'N' only.  Its
 * local rows are the rank's target cluster (get_local_offset /
 * get_local_size, hmatrix.hpp:175-176, set at :320-321). */
int htgpu_hmatrix_set_local_rank(htgpu_hmatrix h, int rank);

/* Right-hand-side buckets (no counterpart in the reference): products with
 * mu right-hand sides (1 <= mu <= 8) run padded with zero columns to
 * mu_run (mu <= mu_run <= 8), one pass over the factors, instead of one
 * pass per group of 4, 2 and 1; mu_run = 0 runs them unpadded.
 * htgpu_hmatrix_autotune(h, mu, ...) sets the faster for mu. */
int htgpu_hmatrix_set_rhs_bucket(htgpu_hmatrix h, int mu, int mu_run);
int htgpu_hmatrix_get_rhs_bucket(htgpu_hmatrix h, int mu, int *mu_run);

/* Reduced-precision products with 4 or more right-hand sides off the tensor
 * cores: on != 0 applies the dense FP64 chunks first in the double-float
 * many-right-hand-side kernel and the FP32 / BF16 chunks after them in the
 * streamed phase-2 kernel; 0 streams every chunk through the one kernel.
 * Results agree within the storage policy's tolerance; the autotuner picks.
 * No counterpart in the reference. */
int htgpu_hmatrix_set_phase2_dense_split(htgpu_hmatrix h, int on);
int htgpu_hmatrix_get_phase2_dense_split(htgpu_hmatrix h, int *on);
int htgpu_hmatrix_local(htgpu_hmatrix h, int *rank, int *local_offset, int *local_size);

/* Replaces HMatrix::mymvprod_global_to_local(in, out, mu)
 * (hmatrix.hpp:844-911), the product behind mymvprod_local_to_local
 * (:980-996) and HPDDM's GMV (wrappers/wrapper_hpddm.hpp:41-83): `in` is
 * the whole input in cluster numbering (nb_cols x mu, column-major: what
 * local_to_global_source all-gathers from the ranks' local parts,
 * hmatrix.hpp:963-977), `out` the handle's local rows (local_size x mu,
 * column-major).  The same as htgpu_hmatrix_mvprod with
 * HTGPU_GLOBAL_TO_LOCAL; flags may add HTGPU_HOST_PTRS.  htool's buffers
 * are row-major for mu > 1; these are column-major like every product
 * here (include/htool_gpu.hpp transposes for htool's callers). */
int htgpu_hmatrix_mvprod_global_to_local(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, void *stream);

/* nb_rows / nb_cols, get_nlrmat / get_ndmat (hmatrix.hpp:173-187). */
int htgpu_hmatrix_sizes(htgpu_hmatrix h, int *nr, int *nc, int *nlr, int *ndense);

/* Leaf descriptors (same layout as htgpu_hmatrix_set_leaves), sorted by
 * (offset_i, offset_j) like HMatrix's MyComputedBlocks (hmatrix.hpp:494-500). */
int htgpu_hmatrix_get_leaves(htgpu_hmatrix h, int *lr_desc, int *d_desc);

/* Factors and dense blocks in htool's layouts (see htgpu_hmatrix_set_leaves). */
int htgpu_hmatrix_get_factors(htgpu_hmatrix h, double *uv, double *dense);

/* get_infos (hmatrix.hpp:223, keys of ComputeInfos, :739-841) plus the GPU
 * assembly counters, as "key=value\n" lines.  Returns the needed size in
 * *len when buf is NULL or too small. */
int htgpu_hmatrix_infos(htgpu_hmatrix h, char *buf, int *len);

/* Bytes of one FP64 product: stored factors and dense blocks, plus the
 * input/output vectors and the two permutations for mu right-hand sides. */
int htgpu_hmatrix_product_bytes(htgpu_hmatrix h, int mu, long long *bytes);

/* Number of this library's kernels the last product launched. */
int htgpu_hmatrix_last_launches(htgpu_hmatrix h, int *launches);

/* Timing breakdown of `reps` products with mu right-hand sides on the
 * handle's stream (device-resident input), measured with CUDA events between
 * the launches: ms[0] gather, ms[1] low-rank V-side (phase 1), ms[2]
 * U-side + dense (phase 2), ms[3] per-cluster sums and scatter, ms[4] whole
 * product; averages per product.  The counterpart of the timing htool accumulates in its infos map
 * (nb_mat_vec_prod / total_time_mat_vec_prod, hmatrix.hpp:1180-1181). */
int htgpu_hmatrix_profile(htgpu_hmatrix h, int mu, int reps, float *ms);

/* Algorithmic bytes of the same four steps with the current storage (no
 * counterpart in the reference): bytes[0] gather (x read twice, gathered
 * copies written), bytes[1] phase 1 (V-side factors, partial sums written),
 * bytes[2] phase 2 (U-side and dense blocks, column indices, cluster sums
 * written), bytes[3] final sums (cluster sums read, y written, perm). */
int htgpu_hmatrix_phase_bytes(htgpu_hmatrix h, int mu, long long *bytes);

/* How the FP64 product shares its work between the FP64 pipe (DFMA) and the
 * FP32/INT pipes (exact double-float emulation, ~2^-46 relative per term):
 * phase1_dfma_permille of the low-rank V-side elements and
 * phase2_dfma_permille of the U-side/dense elements use DFMA.  With a reduced
 * precision set (htgpu_hmatrix_set_precision), the call sets and reads the split
 * of that product's dense blocks, which stay FP64 (phase2_dfma_permille; the
 * phase-1 share is kept for the FP64 product).  Each precision keeps its own
 * split; defaults 0 / 350 (FP64) and 0 (reduced-precision dense blocks),
 * what the autotuner picks on Laplace spheres.  No counterpart in the
 * reference (its BLAS calls decide this, include/htool/types/matrix.hpp:320-383). */
int htgpu_hmatrix_set_fp64_split(htgpu_hmatrix h, int phase1_dfma_permille, int phase2_dfma_permille);
int htgpu_hmatrix_get_fp64_split(htgpu_hmatrix h, int *phase1_dfma_permille, int *phase2_dfma_permille);

/* Phase 1 (the V-side sums of every low-rank leaf) with one or two
 * right-hand sides: HTGPU_PHASE1_TILES (one warp per tile, DFMA and emulated
 * tiles as two concurrent kernels) or HTGPU_PHASE1_STREAM (consecutive tile
 * chunks staged into shared memory by a producer warp with bulk copies and
 * shared by the CTA's consumer warps, the default).  Reduced-precision
 * products with 3 or more right-hand sides off the tensor cores take, in
 * HTGPU_PHASE1_STREAM, the tiles on the same x rows stacked into blocks of
 * 128 columns with one thread per column.  Results agree within the
 * storage policy's tolerance; the autotuner picks one.  No counterpart in
 * the reference. */
#define HTGPU_PHASE1_TILES 0
#define HTGPU_PHASE1_STREAM 1
/* as HTGPU_PHASE1_STREAM, and reduced-precision products with 8 or more
 * right-hand sides take the TF32 tcgen05 phase 1 at any epsilon (the
 * tensor-core phase 2 stays reserved to epsilon >= 1e-5).  Below epsilon
 * 1e-5 the tensor cores' FP32 accumulation can put a right-hand side beyond
 * epsilon from FP64 (1.4e-6 on a 400 000-point sphere at 1e-6), so the
 * autotuner never picks this mode; it keeps it when set. */
#define HTGPU_PHASE1_TENSOR 2
int htgpu_hmatrix_set_phase1_mode(htgpu_hmatrix h, int mode);
int htgpu_hmatrix_get_phase1_mode(htgpu_hmatrix h, int *mode);

/* Pre-split FP64 data for the FP32-pipe emulation (on by default): FP64
 * products keep a second copy of the data their emulated chunks read as
 * (hi, lo) float pairs, so the kernels read the pairs instead of splitting
 * every double again -- the V-side factors when every phase-1 tile is
 * emulated (streamed phase 1), and the emulated phase-2 chunks.  Costs those
 * bytes once more in device memory while the FP64 policy is set (bytes:
 * the current size); results are bitwise the same either way.  No
 * counterpart in the reference. */
int htgpu_hmatrix_set_presplit(htgpu_hmatrix h, int on);
int htgpu_hmatrix_get_presplit(htgpu_hmatrix h, int *on, long long *bytes);

/* Phase 2 (the U-side and dense blocks, per row chunk): HTGPU_PHASE2_WARP
 * (every warp streams its own chunks, claiming ranges of row chunks) or
 * HTGPU_PHASE2_PRODUCER (a producer warp per CTA claims units of row chunks
 * and feeds its consumer warps, the default).  Bitwise equal results (the same per-row
 * summation order); the autotuner picks one.  No counterpart in the
 * reference. */
#define HTGPU_PHASE2_WARP 0
#define HTGPU_PHASE2_PRODUCER 1
int htgpu_hmatrix_set_phase2_mode(htgpu_hmatrix h, int mode);
int htgpu_hmatrix_get_phase2_mode(htgpu_hmatrix h, int *mode);

/* Tensor-core kernels of reduced-precision products with at least 8
 * right-hand sides on H-matrices with epsilon >= 1e-5: HTGPU_TC_MMA_SYNC
 * (warp-level mma.sync TF32 in both phases, one warp per tile or row chunk),
 * HTGPU_TC_TCGEN05 (the default: phase 1 on tcgen05.mma with tensor-memory
 * accumulators, the tiles that share their x rows stacked into GEMMs of up
 * to 128 columns; phase 2 on mma.sync) or HTGPU_TC_TCGEN05_BOTH (phase 2 on
 * tcgen05 as well, four row chunks to one 128-row accumulator).  Results
 * agree within FP32 accumulation.  No counterpart in the reference. */
#define HTGPU_TC_MMA_SYNC 0
#define HTGPU_TC_TCGEN05 1
#define HTGPU_TC_TCGEN05_BOTH 2
int htgpu_hmatrix_set_tensor_core_mode(htgpu_hmatrix h, int mode);
int htgpu_hmatrix_get_tensor_core_mode(htgpu_hmatrix h, int *mode);

/* The tcgen05 phase 1 reading its A operand from a second copy of the
 * low-rank factors, laid out once for the tensor cores (per block of up to
 * 128 stacked columns and 32 source rows: the TF32 hi and lo parts in the
 * MMA's shared-memory layout, 32 KB), brought into shared memory by one bulk
 * copy a slab instead of being decoded and split by the threads.  Costs the
 * copy's memory (*bytes, 0 while off or in FP64); bitwise the same sums.
 * Off by default; htgpu_hmatrix_autotune tries it where the tcgen05 phase 1
 * runs and the copy fits in half the free memory.  No counterpart in the
 * reference. */
int htgpu_hmatrix_set_tensor_core_arena(htgpu_hmatrix h, int on);
int htgpu_hmatrix_get_tensor_core_arena(htgpu_hmatrix h, int *on, long long *bytes);

/* Products with 8 or more right-hand sides on the BF16 tensor cores by
 * exact digit slicing (the Ozaki scheme): every factor column, panel row,
 * right-hand side and coefficient set is scaled by a power of two and cut
 * into base-128 digits (8 planes for FP64 data: 54 bits, FP64-grade sums;
 * 4 for reduced-precision factors: 26 bits, at any epsilon), the plane
 * products are exact integer MMAs, the read-out sums them exactly in
 * 128-bit integers.  FP64 storage: both phases (replacing the double-float
 * kernels); reduced storage: phase 1, and the dense FP64 blocks of phase 2
 * where the dense blocks go first.  Costs a copy of the factors cut into
 * planes (*bytes; 0 while off); on after a build follows it and precision
 * changes.  Off by default; htgpu_hmatrix_autotune tries it where the
 * planes fit in half the free memory.  No counterpart in the reference (its
 * gemm calls, types/matrix.hpp:346, 380). */
int htgpu_hmatrix_set_digit_planes(htgpu_hmatrix h, int on);
int htgpu_hmatrix_get_digit_planes(htgpu_hmatrix h, int *on, long long *bytes);

/* Test support, no counterpart in the reference: d (128 x 64) = a (128 x
 * 32) b (32 x 64), row-major host arrays, computed on CUDA device `device`
 * by the tcgen05 path of the tensor-core kernels (the same shared-memory
 * layout, descriptors, three-term TF32 products and tensor-memory read-out),
 * so that path can be checked on its own. */
int htgpu_debug_tc_gemm(int device, const float *a, const float *b, float *d);

/* Test support, no counterpart in the reference: d (128 x mu) = a (128 x K)
 * b (K x mu), row-major FP64 host arrays, K <= 256, computed on CUDA device
 * `device` by the digit-plane path of the tensor-core phase 1 (the FP64
 * products cut into S = 8 or 4 BF16 digit planes, exact MMA sums, integer
 * read-out): one stacked block through the plane packing, the input's
 * exponents and planes and the phase-1 kernel -- the one for inputs cut into
 * planes once, or (staged != 0) the one of wide inputs. */
int htgpu_debug_oz_gemm(int device, int S, int K, int mu, int staged, const double *a, const double *b, double *d);

/* Status word of the product kernels' bounded waits: 0, or 1/2/3 when a
 * wait for a pipeline stage ran out, 4 when a wait of the tensor-core
 * kernels did (the product's result is then not valid).  Synchronises the H-matrix's stream.  Host-pointer products check
 * it themselves and fail.  No counterpart in the reference. */
int htgpu_hmatrix_device_status(htgpu_hmatrix h, int *status);
/* Clears the status word (after a reported expiry), synchronising the
 * H-matrix's stream.  No counterpart in the reference. */
int htgpu_hmatrix_reset_status(htgpu_hmatrix h);

/* Test support, no counterpart in the reference: on CUDA device `device`,
 * the limit of every bounded wait of the product kernels in SM clock cycles
 * (default 4e9, about 2 s) and the index of one chunk of the producer-fed
 * phase 2 (HTGPU_PHASE2_PRODUCER) whose bulk copies are left out, so that
 * its consumer's wait runs out (-1, the default: none).  Lets a test see
 * the kernels give up, report status 2 / 3 and return; restore the
 * defaults afterwards. */
int htgpu_debug_set_waits(int device, long long cycles, long long skip_chunk);

/* Autotuner: times `reps` products with mu right-hand sides on this
 * H-matrix and keeps the fastest configuration for the current storage
 * policy -- with FP64 factors the phase-1 mode and the DFMA/emulation
 * split, with reduced-precision factors the phase-1 mode; *best_ms is its
 * time per product.  Replaces nothing
 * upstream (htool has no tuning). */
int htgpu_hmatrix_autotune(htgpu_hmatrix h, int mu, int reps, float *best_ms);

/* Storage of the low-rank factors used by the products (no counterpart in
 * the reference, which is FP64/complex128 throughout): HTGPU_PREC_FP64,
 * HTGPU_PREC_FP32, HTGPU_PREC_MIXED (per column: FP32 for the leading ACA
 * crosses, BF16 for those whose bound max|u_k| max|v_k| sqrt(m n) is below
 * tau * epsilon * (leaf bound) / 2^-9) or HTGPU_PREC_BF16.  Every column is
 * stored divided by its maximum, with the product of the two maxima kept
 * in FP64; dense leaves stay FP64; all sums are FP32 or wider.  The FP64
 * factors are kept, so the policy can be switched back at any time. */
#define HTGPU_PREC_FP64 0
#define HTGPU_PREC_FP32 1
#define HTGPU_PREC_MIXED 2
#define HTGPU_PREC_BF16 3
int htgpu_hmatrix_set_precision(htgpu_hmatrix h, int policy, double tau);
/* Active policy, bytes of factors + dense blocks one product reads, and the
 * number of FP32 and BF16 low-rank columns. */
int htgpu_hmatrix_precision_info(htgpu_hmatrix h, int *policy, long long *stored_bytes, long long *fp32_columns, long long *bf16_columns);

/* No counterpart in the reference.  The product of htgpu_hmatrix_mvprod for
 * device pointers, but allocation-free: it never calls cudaMalloc, cudaFree
 * or any other allocating routine, for callers that cannot let a library
 * allocate device memory mid-run -- e.g. a process whose framework has
 * already reserved the GPU's memory for its own pool, or a solver driving
 * the product from a hot loop.  Its working memory is one fixed 16 MiB
 * array per device inside the library (2^21 doubles); a product needs
 * 2 * nb_cols * mu (each half rounded up to 32) + 32 + (phase-1 partial sums
 * + per-cluster partial-sum rows) * mu doubles, and larger requests fail
 * with HTGPU_ERR_INVALID.  The array is made resident, and its device
 * address looked up (cudaGetSymbolAddress, with that device current), when
 * the first H-matrix is created on a device -- before a caller's memory
 * pool is likely to hold the GPU -- and it stays until the process exits;
 * if that lookup failed, the first call here repeats it, so that call should
 * then come before any stream capture.  Every call shares the one array,
 * whose contents persist between calls: calls that may overlap on the GPU
 * (different streams, or different handles on one device) race with each
 * other and must be serialised by the caller.  The call also uses the
 * handle's own status word and work tickets, like htgpu_hmatrix_mvprod:
 * any two products of one handle that may overlap on the GPU, this one or
 * the regular ones, must be serialised.  Like the device-pointer
 * htgpu_hmatrix_mvprod, it returns before the product ran and does not read
 * the status of the kernels' bounded waits: after synchronising, a caller
 * that must know the result is valid reads htgpu_hmatrix_device_status.
 * in/out: device memory, column-major, user numbering; ordered on `stream`
 * (NULL = the handle's own stream). */
int htgpu_hmatrix_mvprod_noalloc(htgpu_hmatrix h, const double *in, double *out, int mu, void *stream);

/* ---- ACA rank predictor (no counterpart in the reference) ------------------
 * A 10 -> 64 -> 64 -> 1 perceptron (FP32, ReLU) that predicts from an
 * admissible block's geometry how many ACA crosses the block needs; trained
 * on the GPU on (features, crosses) pairs that partialACA itself produced.
 * An H-matrix build can use it to size every block's first ACA attempt;
 * partialACA's own stopping test still decides each rank, and a block whose
 * scratch runs out is re-run with more, so the H-matrix is the same with or
 * without the predictor. */
int htgpu_mlp_num_params(void); /* W1[64][10], b1[64], W2[64][64], b2[64], W3[64], b3 */
int htgpu_mlp_create(int device, unsigned long long seed, htgpu_mlp *out); /* Glorot-uniform weights from seed */
int htgpu_mlp_destroy(htgpu_mlp m);
int htgpu_mlp_set_params(htgpu_mlp m, const float *params); /* host; resets the optimiser */
int htgpu_mlp_get_params(htgpu_mlp m, float *params);
/* Adam (0.9, 0.999) on the mean squared error over minibatches of `batch`
 * shuffled samples (features: n x 10 row-major, host); loss_per_epoch
 * (optional, `epochs` floats): the loss over all samples after each epoch. */
int htgpu_mlp_train(htgpu_mlp m, const float *features, const float *ranks, int n, int epochs, int batch, float lr, unsigned long long seed, float *loss_per_epoch);
/* Gradient (htgpu_mlp_num_params floats) and value of the mean squared error
 * over the n samples taken as one batch. */
int htgpu_mlp_gradient(htgpu_mlp m, const float *features, const float *ranks, int n, float *grad, float *loss);
int htgpu_mlp_predict(htgpu_mlp m, const float *features, int n, float *ranks);
/* The 10 features of a block (sizes M x N, cluster radii and centres). */
int htgpu_block_features(int M, int N, double rad_t, double rad_s, const double *ctr_t, const double *ctr_s, double epsilon, int kernel_id, float *features);
/* Size the first ACA attempt of every block of later builds from the
 * predictor: max(4, ceil(prediction * (1 + margin)) + 2) crosses, the
 * largest profitable rank for predictions of 60 and above; NULL restores
 * the fixed first attempt of 48.  The predictor must outlive those builds. */
int htgpu_hmatrix_set_rank_predictor(htgpu_hmatrix h, htgpu_mlp m, double margin);
/* Device bytes of ACA scratch one slice of blocks may use (0: 60% of the
 * free memory at each round). */
int htgpu_hmatrix_set_aca_budget(htgpu_hmatrix h, long long bytes);
/* (features, crosses needed) of every block the last build's partialACA
 * decided: its rank, or for a rejected block the largest profitable rank.
 * With features == ranks == NULL only *count is set. */
int htgpu_hmatrix_aca_samples(htgpu_hmatrix h, float *features, float *ranks, int capacity, int *count);

/* ---- batched products (no counterpart in the reference) --------------------
 * Many H-matrices, each with its own device input and output (column-major,
 * user numbering, mu right-hand sides), applied by one CUDA-graph launch.
 * htgpu_batch_capture runs every product once, then records them all, spread
 * over up to nstreams concurrent streams (largest first); each launch
 * replays the graph and reads / writes the buffers given at add time.  The
 * H-matrices and buffers must outlive the batch; adding an entry drops the
 * captured graph.  stream NULL: the batch's own stream. */
int htgpu_batch_create(int device, htgpu_batch *out);
int htgpu_batch_destroy(htgpu_batch b);
int htgpu_batch_add(htgpu_batch b, htgpu_hmatrix h, const double *in, double *out, int mu, int *index);
/* The same with flags: HTGPU_CLUSTER_NUMBERING makes the entry a product in
 * cluster (local) numbering, htool's mymvprod_local_to_local on one rank
 * (hmatrix.hpp:980-996; mvprod_local_to_local after set_use_permutation(false),
 * :1185-1274): what HPDDM's GMV calls in a Krylov loop
 * (wrappers/wrapper_hpddm.hpp:41-83); HTGPU_GLOBAL_TO_LOCAL the product of
 * htgpu_hmatrix_mvprod_global_to_local (a rank's part of a multi-rank
 * product, its input already gathered).  Device pointers only. */
int htgpu_batch_add_flags(htgpu_batch b, htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, int *index);
int htgpu_batch_capture(htgpu_batch b, int nstreams, long long *graph_nodes);
int htgpu_batch_launch(htgpu_batch b, void *stream);
int htgpu_batch_sync(htgpu_batch b);

/* Row partition for a product over several GPUs (the distribution of
 * include/htool/types/hmatrix.hpp:964-977, 1103: every part owns a range of
 * target rows in cluster numbering and computes them completely; x is
 * all-gathered before and y after).  leaves: (offset_i, m, stored bytes) per
 * leaf; cuts: nparts + 1 row offsets, never inside a leaf's rows, balancing
 * the bytes.  Host only. */
int htgpu_partition_rows(int nleaves, const long long *leaves, int nr, int nparts, int *cuts);

/* y = H^T x (HMatrix::mvprod_transp_global_to_global,
 * include/htool/types/hmatrix.hpp:1277-1455), user numbering, mu
 * right-hand sides (in: nr * mu, out: nc * mu).  The first call builds a
 * transposed copy of the leaves inside the handle (one pass through host
 * memory, as much device memory again); later calls reuse it and follow the
 * handle's storage policy.  flags: HTGPU_HOST_PTRS or 0. */
int htgpu_hmatrix_mvprod_transp(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned flags, void *stream);

/* Cluster trees in htool's CSV pair (VirtualCluster::save_cluster /
 * read_cluster, include/htool/clustering/cluster.hpp:433-583):
 * <name>_permutation.csv and <name>_tree.csv, radii and centres with 6
 * significant digits as htool writes them.  Host only. */
int htgpu_cluster_save(htgpu_cluster c, const char *name);
int htgpu_cluster_read(const char *perm_file, const char *tree_file, htgpu_cluster *out);

/* Binary dump of an assembled H-matrix (leaf lists and factors in htool's
 * layout, sizes, permutation hashes, symmetry / UPLO and the complex flag in
 * the header; no counterpart in the reference) and its reload into a handle
 * of the same type on the same cluster trees, e.g. to reuse a large build.
 * A symmetric H-matrix dumps its stored triangle; the reload takes the
 * dump's symmetry and makes the twins again (bitwise the same products). */
int htgpu_hmatrix_save(htgpu_hmatrix h, const char *path);
int htgpu_hmatrix_load(htgpu_hmatrix h, const char *path);

/* htool's leaf map, HMatrix::save_plot (include/htool/types/hmatrix.hpp:1696-1712):
 * writes <outputname>_0.csv (one rank) with "nr,nc" and one line
 * "offset_i,size_i,offset_j,size_j,rank" per leaf, dense leaves first with
 * rank -1, in htool's leaf order; the file tools/plot_hmatrix.py reads. */
int htgpu_hmatrix_save_plot(htgpu_hmatrix h, const char *outputname);

#ifdef __cplusplus
}
#endif
#endif
