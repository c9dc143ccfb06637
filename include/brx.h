/*
 * brx.h — C ABI of the GB300 query path for brille's BrillouinZoneTrellis3.
 *
 * The reference answers `ir_interpolate_at` / `interpolate_at` on the host
 * (src/bz_trellis.hpp:113-196).  This ABI takes the same question to one
 * GB300: a caller that already holds a constructed Brillouin zone and trellis
 * flattens them into a brx_geometry (plain pointers and sizes), uploads it
 * once with brx_create, fills vertex data with brx_fill and then asks for
 * interpolated values and vectors at any number of Q points.
 *
 * Every function returns a brx_status; none throws and none takes a torch or
 * C++ type.  Pointers to Q and to outputs may be host or device memory: host
 * buffers are staged through pinned memory in chunks on the handle's streams,
 * device buffers are used in place.  The status enum mirrors the reference's
 * error messages (src/bz_trellis.hpp:165-169, src/bz_move.cpp:158,288-294,
 * src/trellis_poly.hpp:345-350, src/trellis_node.hpp:593-610,
 * src/interpolator.hpp:400-426); brx_last_error returns the message text.
 */
#ifndef BRX_H
#define BRX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BRX_ABI_VERSION 1

typedef enum brx_status {
  BRX_OK = 0,
  BRX_ERR_INVALID_ARGUMENT = 1,
  BRX_ERR_CUDA = 2,
  BRX_ERR_NOT_FILLED = 3,        /* "The interpolation data must be filled before interpolating." */
  BRX_ERR_MOVE_FAILED = 4,       /* "Not all points inside Brillouin zone" (bz_move.cpp:149-159) */
  BRX_ERR_OUTSIDE_IR = 5,        /* "Q = ... is outside of the irreducible BrillouinZone" (bz_move.cpp:288-294) */
  BRX_ERR_NOT_FOUND = 6,         /* "interpolate_at failed to find N points" (trellis_poly.hpp:345-350) */
  BRX_ERR_NULL_NODE = 7,         /* "Attempting to access null node at index" (trellis_node.hpp:593-610) */
  BRX_ERR_UNSUPPORTED = 8,       /* "LengthUnit, RotatesLike combination not implemented" (interpolator.hpp:400-426) */
  BRX_ERR_IMPOSSIBLE = 9,        /* "This shouldn't be possible" (trellis_node.hpp:298-300) */
  BRX_ERR_OUT_OF_MEMORY = 10,
  BRX_ERR_TIMEOUT = 11           /* a bounded device-side wait ran out */
} brx_status;

/* Node types of the trellis, reference NodeType (src/enums.hpp:73). */
enum { BRX_NODE_NULL = 0, BRX_NODE_CUBE = 1, BRX_NODE_POLY = 2 };

/* RotatesLike and LengthUnit codes as the reference's fill() decodes them
 * (wrap/_interpolator.hpp:28-45). */
enum { BRX_ROT_VECTOR = 0, BRX_ROT_PSEUDOVECTOR = 1, BRX_ROT_GAMMA = 2 };
enum { BRX_LU_NONE = 0, BRX_LU_ANGSTROM = 1, BRX_LU_INVERSE_ANGSTROM = 2,
       BRX_LU_REAL_LATTICE = 3, BRX_LU_RECIPROCAL_LATTICE = 4 };

/* Element types. */
enum { BRX_F64 = 0, BRX_C128 = 1, BRX_F32 = 2, BRX_C64 = 3, BRX_BF16 = 4 };

/* Storage precision of vertex data on the device (brx_fill). */
enum { BRX_STORE_F64 = 0,  /* as given: float64 / complex128, FP64 arithmetic */
       BRX_STORE_F32 = 1,  /* float32 / complex64, FP32 arithmetic           */
       BRX_STORE_BF16 = 2  /* eigenvectors as bfloat16 pairs, eigenvalues float32; FP32 arithmetic */ };

/* Query flags (brx_ir_interpolate_at / brx_interpolate_at). */
#define BRX_FLAG_NO_MOVE   0x1u  /* do_not_move_points: Q already irreducible / in the first zone */
#define BRX_FLAG_OUT_F32   0x2u  /* write float32 / complex64 outputs instead of the input dtype  */
#define BRX_FLAG_ASYNC     0x4u  /* return without synchronising; errors are read later with
                                    brx_sync.  Q and outputs in device memory, or in page-locked
                                    host memory (cudaHostAlloc / cudaHostRegister): then the
                                    outputs are complete only after brx_sync or an event recorded
                                    on the stream behind the call.  With pageable host memory the
                                    call synchronises as without the flag.  Calls may be queued on
                                    several streams; they share one error word until brx_sync,
                                    which waits for all of them. */
/* Diagnostic, no counterpart in the reference: the first bounded device
 * wait of every warp of the FP32/BF16 vectors gather, and of every slot of
 * the tensor-core residual network, waits on a barrier that nothing
 * completes, so it gives up after about a millisecond.  The kernels then
 * take their error path (error flag, copies in flight drained, tensor
 * memory released) and the call returns BRX_ERR_TIMEOUT.  For tests of that
 * path only: the outputs of such a call are incomplete. */
#define BRX_FLAG_TEST_TIMEOUT 0x100u

/*
 * Everything the query path reads, flattened.  All arrays are row-major and
 * are copied to the device by brx_create; the caller keeps ownership.
 * Coordinates are Cartesian 1/Å unless stated.
 */
typedef struct brx_geometry {
  /* -- lattices: the reference's BrillouinZone::_outer and _inner -- */
  double outer_B[9];          /* rows b1,b2,b3 of the (conventional) reciprocal basis: xyz = hkl · B */
  double prim_B[9];           /* rows of the primitive reciprocal basis */
  int32_t to_prim_6Pt[9];     /* primitive hkl = (6Pᵀ · hkl) / 6   (src/transform.hpp:168-191) */
  int32_t from_prim_invPt[9]; /* conventional hkl = (P⁻¹)ᵀ · primitive hkl (src/transform.hpp:212-221) */
  int32_t is_primitive;       /* 1: conventional == primitive, no transform (PrimitiveTransform::does_nothing) */

  /* -- first Brillouin zone, one entry per face (BrillouinZone::moveinto, src/bz_move.cpp:123-141) -- */
  int32_t n_faces;
  const double* face_abc;     /* n_faces × 9: points a, b, c on the face; orient3d(a,b,c,0) > 0 */
  const double* face_normal;  /* n_faces × 3: unit outward normal */
  const int32_t* face_tau;    /* n_faces × 3: primitive-lattice τ whose bisector the face is */
  const double* face_tau_len; /* n_faces: |τ| */

  /* -- irreducible wedge (BrillouinZone::_inside_wedge_outer, src/bz.hpp:757-763) -- */
  int32_t n_wedge;
  const double* wedge_normal; /* n_wedge × 3 */
  int32_t wedge_le_ge;        /* 0: inside when every n·q ≥ 0; 1: when every n·q ≥ 0 or every n·q ≤ 0 */

  /* -- point group (BrillouinZone::get_pointgroup_symmetry, src/bz.hpp:743-746) -- */
  int32_t n_ops;
  const int32_t* ops;         /* n_ops × 9: direct-lattice integer matrices W; q_ir = Wᵀ q */
  const int32_t* op_inverse;  /* n_ops: index of W⁻¹ (PointSymmetry::get_inverse_index) */
  int32_t identity;           /* PointSymmetry::find_identity_index */
  double lattice_to_xyz[9];   /* direct lattice: columns are a1,a2,a3 in Å (to_xyz(angstrom)) */
  double lattice_from_xyz[9]; /* its inverse */

  /* -- trellis (PolyTrellis, src/trellis_poly.hpp; NodeContainer, src/trellis_node.hpp) -- */
  int32_t n_knots[3];
  const double* knots[3];     /* n_knots[d] bin edges along x, y, z */
  int64_t n_nodes;            /* Π (n_knots[d]-1); linear index i + nx(j + ny k) */
  const int32_t* node_type;   /* n_nodes: BRX_NODE_* */
  const int32_t* node_index;  /* n_nodes: index into cube or poly nodes */
  int32_t n_cube;
  const int32_t* cube_vertices;   /* n_cube × 8, order (000)(100)(110)(010)(101)(001)(011)(111) */
  int32_t n_poly;
  const int32_t* poly_tet_offset; /* n_poly + 1 */
  int64_t n_tets;
  const int32_t* tet_vertices;    /* n_tets × 4, positively oriented */
  const double* tet_sphere;       /* n_tets × 4: circumsphere centre x,y,z and radius */
  const double* tet_volume;       /* n_tets */
  int64_t n_vertices;
  const double* vertex_xyz;       /* n_vertices × 3 */

  /* -- Γ table for phonon eigenvectors (GammaTable, src/phonon.hpp:91-194) -- */
  int32_t n_atoms;
  const int32_t* gamma_F0;        /* n_atoms × n_ops: l = F0(k, r) */
  const int32_t* gamma_vidx;      /* n_atoms × n_ops: index into gamma_vectors */
  int32_t n_gamma_vectors;
  const double* gamma_vectors;    /* n_gamma_vectors × 3: R⁻¹ r_l − r_k, fractional direct */

  /* -- approx_float::Config (src/approx_config.hpp:17) -- */
  double float_tolerance;         /* config.reciprocal, default 1e-12 */
  int32_t digit;                  /* config.digit, default 1000 */
} brx_geometry;

/* Vertex data of one interpolator (the values or the vectors of a
 * DualInterpolator, src/interpolatordual.hpp; decoded as in
 * wrap/_interpolator.hpp:13-110). */
typedef struct brx_data {
  const void* data;               /* n_vertices × n_branches × span elements (host or device) */
  int32_t dtype;                  /* BRX_F64, BRX_C128, BRX_F32 or BRX_C64 */
  int32_t n_branches;             /* B */
  int32_t elements[3];            /* scalars, vector elements (3 per vector), matrix elements (9 per matrix) */
  int32_t rotates_like;           /* BRX_ROT_* */
  int32_t length_unit;            /* BRX_LU_* */
} brx_data;

/* Per-q record of the locate stages, for index-level parity checks. */
typedef struct brx_locate_out {
  double* q_ir;                   /* n × 3: irreducible (or first-zone) q, r.l.u. */
  int32_t* tau;                   /* n × 3: conventional τ with Q = Rᵀ q + τ (may be NULL) */
  int32_t* rot;                   /* n × 2: R index and R⁻¹ index (may be NULL) */
  int32_t* node;                  /* n × 2: node linear index and tetrahedron index (−1 for cube nodes) */
  int32_t* n_weights;             /* n: number of (vertex, weight) pairs */
  int32_t* vertex;                /* n × 8 */
  double* weight;                 /* n × 8 */
  int32_t* status;                /* n: 0 ok, else a brx_status code */
} brx_locate_out;

typedef struct brx_handle brx_handle;

/* Upload the geometry; replaces BrillouinZoneTrellis3 construction as far as
 * the query path is concerned (src/bz_trellis.hpp:56-59). */
brx_status brx_create(const brx_geometry* geometry, int32_t device, brx_handle** out);
void brx_destroy(brx_handle* h);

/* Upload vertex data, replacing fill() (wrap/_common_grid.hpp:26-47,127-147;
 * DualInterpolator::replace_data, src/interpolatordual.hpp:189-195).
 * `vectors` may be NULL for a values-only grid.  storage is BRX_STORE_*. */
brx_status brx_fill(brx_handle* h, const brx_data* values, const brx_data* vectors, int32_t storage);

/* Optional mode-permutation table from sort() (PermutationTable,
 * src/permutation_table.hpp:63-266): keys i*n_vertices+j sorted ascending,
 * each naming one of n_perms permutations of n_branches modes.  Pairs not
 * listed use the identity, as PermutationTable::safe_get does (:193-198). */
brx_status brx_set_permutations(brx_handle* h, int64_t n_keys, const int64_t* keys,
                                const int32_t* perm_ids, int32_t n_perms, const int32_t* perms);

/* sort(): find the mode permutation of every listed vertex pair on the GPU
 * and keep it as the handle's permutation table, replacing
 * DualInterpolator::sort (src/interpolatordual.hpp:398-434) with the cost
 * matrix of cost_matrix/add_cost (:385-396, src/interpolator_cost.tpp:19-61)
 * and an exact assignment where the reference runs LAPJV (:420-434).
 * keys: i*n_vertices+j, strictly increasing, i != j, and j*n_vertices+i
 * listed for every i*n_vertices+j (the reference's permutation keys: every
 * ordered pair of distinct vertices of a cube node or of one tetrahedron,
 * src/trellis_poly_parallel.tpp:485-526).  values_cost / vectors_cost may be
 * NULL for the defaults (functions 0, weights 1).  Costs are FP64 on the
 * stored data (FP32/BF16 storage: on the rounded data).  One vertex pair's
 * rows and cost matrix must fit one CTA's shared memory (about 40·B² bytes
 * for phonon data, B modes of B complex elements: B ≤ 74 with FP64
 * storage, B ≤ 95 with FP32 storage).
 * Synchronous on stream (NULL: the handle's stream).  Invalid keys or cost
 * codes are rejected before the old table is touched; a failure after that
 * (a reverse key missing, a cost matrix without a finite assignment) leaves
 * the handle with no permutation table, as after brx_fill. */
typedef struct brx_sort_cost {
  int32_t scalar_fn;  /* fill's elements[5]: 0, Σ|a−b| (the reference's only scalar cost) */
  int32_t vector_fn;  /* fill's elements[6]: 1 |a−b|, 2 1−|a*·b|², 3 Euclidean angle,
                         4 Hermitian angle, any other: sin² of the Hermitian angle
                         (src/interpolator.hpp:246-300) */
  double weight[3];   /* relative cost of scalar, vector and matrix elements (fill's weights) */
} brx_sort_cost;
brx_status brx_sort(brx_handle* h, int64_t n_keys, const int64_t* keys, const brx_sort_cost* values_cost,
                    const brx_sort_cost* vectors_cost, void* stream);
/* The permutation table as PermutationTable::safe_get reads it
 * (src/permutation_table.hpp:193-198): the handle's n_keys keys and, per key,
 * the permutation of n_branches modes (identity where none is set).
 * n_keys must equal the handle's count (0 after brx_fill). */
brx_status brx_get_permutations(brx_handle* h, int64_t n_keys, int64_t* keys_out, int32_t* perms_out);
/* Number of permutation keys the handle holds. */
int64_t brx_permutation_count(const brx_handle* h);

/* ir_interpolate_at (src/bz_trellis.hpp:155-196; wrap/_common_grid.hpp:276-300).
 * Q: n × 3 float64 in conventional r.l.u.; values_out: n × B_v × span_v and
 * vectors_out: n × B_c × span_c in the input dtype (or float32/complex64 with
 * BRX_FLAG_OUT_F32).  stream is a cudaStream_t or NULL for the handle's own. */
brx_status brx_ir_interpolate_at(brx_handle* h, const double* Q, int64_t n,
                                 void* values_out, void* vectors_out,
                                 uint32_t flags, void* stream);

/* Coherent one-phonon structure factor of the interpolated modes (no
 * counterpart in the reference; the consumer that brille feeds): per q and
 * mode j, S_j = |Σ_k c_k e^{2πi Q·x_k} (Q_c · e_jk)|², with Q_c = Q·B in Å⁻¹
 * (B: rows of the reciprocal basis), e_jk the Γ-rotated Cartesian
 * eigenvector of atom k as brx_ir_interpolate_at returns it, c_k = b_k/√m_k
 * and x_k (fractional, in the lattice of Q's r.l.u.) from brx_set_atoms.
 * The eigenvectors are never written out: values_out as for
 * brx_ir_interpolate_at, sf_out n × B float32.  Needs FP32 or BF16 storage
 * of complex eigenvectors of 1-32 atoms (no other elements) with
 * LengthUnit Å and RotatesLike Γ. */
typedef struct {
  int32_t n_atoms;
  const double* weight;    /* n_atoms: b_k / sqrt(m_k) */
  const double* position;  /* n_atoms × 3, fractional */
} brx_atoms;
brx_status brx_set_atoms(brx_handle* h, const brx_atoms* atoms);
brx_status brx_ir_structure_factor(brx_handle* h, const double* Q, int64_t n, void* values_out, float* sf_out,
                                   uint32_t flags, void* stream);

/* interpolate_at: first-zone move and interpolation, no rotation
 * (src/bz_trellis.hpp:113-129; wrap/_common_grid.hpp:412-440). */
brx_status brx_interpolate_at(brx_handle* h, const double* Q, int64_t n,
                              void* values_out, void* vectors_out,
                              uint32_t flags, void* stream);

/* The locate stages alone (ir_moveinto + node/tetrahedron search) with every
 * intermediate index written out; `ir` selects ir_moveinto (1) or moveinto (0). */
brx_status brx_locate(brx_handle* h, const double* Q, int64_t n, int32_t ir,
                      uint32_t flags, const brx_locate_out* out, void* stream);

/* ---------------------------------------------------------------------
 * Trellis construction on the GPU (reference: PolyTrellis::construct,
 * src/trellis_poly_parallel.tpp:74-482, which classifies the knot grid's
 * cells and tetrahedralises the cells the polyhedron's surface cuts with
 * TetGen).  One thread per cell classifies it from its corners' signed
 * distances to the polyhedron's planes: cube (every corner inside), null
 * (every corner outside one plane) or cut.  One thread per cut cell gathers
 * the corners of the cell ∩ polyhedron (cell corners inside, polyhedron
 * vertices in the cell, cell edges through polyhedron planes, polyhedron
 * edges through cell faces), merges them within tol, and splits the convex
 * polytope into tetrahedra by a fan from its first corner over each facet
 * it does not touch.  Cut cells that span no volume become null nodes.
 * The caller merges the cut cells' corners with the knot points of the
 * cube nodes into one vertex list.
 */
typedef struct brx_trellis_in {
  int32_t n_vertices;
  const double* vertices;     /* polyhedron vertices, n × 3 (Å⁻¹) */
  int32_t n_planes;
  const double* planes;       /* n × 4 (unit normal, offset): inside where n·x + d ≤ tol; no two alike */
  int32_t n_edges;
  const int32_t* edges;       /* n × 2 vertex indices of the polyhedron's edges */
  int32_t n_knots[3];
  const double* knots[3];     /* strictly increasing */
  double tol;                 /* absolute distance tolerance */
  int32_t always_triangulate; /* 1: no cube nodes */
} brx_trellis_in;

typedef struct brx_trellis_cells {
  int64_t n_nodes;
  int32_t* node_type;         /* BRX_NODE_* per node, linear index i + nx(j + ny k) */
  int64_t n_poly;
  int32_t* poly_node;         /* n_poly linear node indices of the POLY nodes, increasing */
  int64_t* point_offset;      /* n_poly + 1 */
  double* points;             /* point_offset[n_poly] × 3 corners of each cut polytope */
  int64_t* tet_offset;        /* n_poly + 1 */
  int32_t* tets;              /* tet_offset[n_poly] × 4, indices into the cell's own corners */
} brx_trellis_cells;

/* Fills *out with arrays this library allocates in host memory; release
 * them with brx_trellis_cells_free.  BRX_ERR_UNSUPPORTED if a cut cell has
 * more than 128 corners or 512 tetrahedra, or the polyhedron more than 64
 * planes; BRX_ERR_IMPOSSIBLE if the write pass disagrees with the count pass. */
brx_status brx_trellis_cells_build(const brx_trellis_in* in, int32_t device, brx_trellis_cells* out);
void brx_trellis_cells_free(brx_trellis_cells* out);

/* ir_interpolate_at for callers that must not allocate device memory while
 * they run: serving loops that cannot take the device-wide synchronisation
 * of cudaMalloc/cudaFree inside a request, and plugins of host frameworks
 * whose own caching pool owns the device memory.  No counterpart in the
 * reference.  All per-q scratch lives in one fixed __device__ array of this
 * library (about 14 MB on every device that loads it, kept until exit), so a
 * call allocates nothing.  Limits: Q and outputs must be device memory of the
 * handle's device; n ≤ BRX_NOALLOC_MAX_Q (larger n is rejected with
 * BRX_ERR_INVALID_ARGUMENT).  The first call on a device looks up the
 * array's address and loads the kernels; make it before any stream capture.
 * Calls share the array, which keeps the last call's contents: calls that
 * overlap on the GPU race and must be serialised. */
#define BRX_NOALLOC_MAX_Q 65536
brx_status brx_ir_interpolate_at_noalloc(brx_handle* h, const double* Q, int64_t n,
                                         void* values_out, void* vectors_out,
                                         uint32_t flags, void* stream);

/* ---------------------------------------------------------------------
 * Learned eigenvalue residual.  No counterpart in the reference: a small
 * MLP (d_in → 128 → 128 → 128 → n_out, GELU, bf16 weights, FP32
 * accumulation) predicts per mode the exact eigenvalue minus its trellis
 * interpolation, so that a coarser trellis serves the accuracy of a finer
 * one.  Feature rows are built on the GPU from locate records:
 *   0-2 position of q in its node cell; 3-10 the weights of the vertex
 *   slots; 11 tetrahedron flag; 12 + slot·B + mode the vertex eigenvalues;
 *   12 + 8B + mode the interpolated eigenvalues; 12 + 9B + 0..2 the
 *   position of q in the trellis's bounding box; 15 + 9B the distance of q
 *   to Γ over the box's longest side; zeros up to d_in;
 * eigenvalues divided by omega_scale.  d_in ≥ 16 + 9B, a multiple of 16,
 * ≤ 512; n_out a multiple of 8, ≤ 64, ≥ n_modes = B.  Parameters are one
 * FP32 vector: W0 (128×d_in, row-major [out][in]), b0, W1, b1, W2, b2,
 * W3 (n_out×128), b3.  Every pointer below except the host params of
 * brx_set_residual_model is a device pointer. */
typedef struct brx_mlp_dims {
  int32_t d_in;
  int32_t n_out;
  int32_t n_modes;
  int32_t flags;  /* BRX_MLP_FP32: training kernels skip the bf16 rounding */
} brx_mlp_dims;
#define BRX_MLP_FP32 0x1

/* Length of the parameter vector, or −1 for invalid dimensions. */
int64_t brx_mlp_param_count(const brx_mlp_dims* d);
/* Floats of workspace that brx_mlp_train_step / brx_mlp_forward need. */
int64_t brx_mlp_workspace_floats(const brx_mlp_dims* d, int64_t batch);

/* Feature rows X (n × d_in) and plain interpolated eigenvalues base (n × B,
 * NaN where the locate failed) from device locate records (every array of
 * `records` set).  stream NULL: the handle's stream, synchronised. */
brx_status brx_mlp_features(brx_handle* h, const brx_locate_out* records, int64_t n, const brx_mlp_dims* d,
                            float omega_scale, float* X, float* base, void* stream);

/* One training step on a batch: forward (weights and activations rounded
 * to bf16 as inference rounds them), mean squared error against T
 * (batch × n_modes) written to *loss, gradients into grads (same layout as
 * params), then, when adam_m/adam_v are given, an Adam update (β 0.9/0.999,
 * ε 1e-8, bias correction with step ≥ 1) of params. */
brx_status brx_mlp_train_step(const brx_mlp_dims* d, float* params, float* grads, float* adam_m, float* adam_v,
                              int32_t step, float lr, const float* X, const float* T, int64_t batch,
                              float* workspace, float* loss, void* stream);

/* Network outputs Y (batch × n_out) in training arithmetic. */
brx_status brx_mlp_forward(const brx_mlp_dims* d, const float* params, const float* X, int64_t batch, float* Y,
                           float* workspace, void* stream);

/* Attach a trained model (host params) to the handle: from now on every
 * query adds res_scale × output to the interpolated eigenvalues, except
 * where that correction exceeds clip in magnitude (clip 0: never), which
 * keeps the plain interpolation.  params NULL detaches the model. */
brx_status brx_set_residual_model(brx_handle* h, const brx_mlp_dims* d, const float* params, float omega_scale,
                                  float res_scale, float clip);

/* ---------------------------------------------------------------------
 * Batched queries over many interpolators (the batched entry point the
 * reference's host would add beside ir_interpolate_at; no counterpart in
 * the reference itself).  Every stage of a batch is one launch over all
 * items: locate, the counting sort of all items' q, the values gather and
 * the vectors gather.  Items may differ in trellis, space group, mode and
 * atom count and q count; they must share the device, the storage kind
 * and complex-ness of their values and of their vectors, whether values
 * are scalar-only, and whether vectors are present.  Handles must outlive
 * the batch and keep their data (no brx_fill in between).  Q and outputs
 * are device buffers with the single-query layouts.
 *
 *   brx_batch_create   plan for n items with n_q[i] q each (ir: 1 for
 *                      ir_interpolate_at, 0 for interpolate_at; flags:
 *                      BRX_FLAG_NO_MOVE, BRX_FLAG_OUT_F32)
 *   brx_batch_set_io   the items' Q and output pointers (host arrays of
 *                      device pointers; vectors NULL without vectors)
 *   brx_batch_run      enqueue the batch on stream: copies and launches
 *                      only, so it can be recorded by a stream capture
 *   brx_batch_capture  record brx_batch_run into a CUDA graph kept by the
 *                      batch; brx_batch_launch replays it (and sees the
 *                      pointers of the latest brx_batch_set_io)
 *   brx_batch_sync     wait for stream; the first failing item's status and
 *                      message (prefixed "item i: "), its index in *failed
 *   brx_batch_tune     time launch-shape candidates on the current I/O with
 *                      CUDA events (locate block size, CTAs per SM, q per
 *                      tile; each gather's kernel and shared-memory budget)
 *                      and keep the fastest; drops a captured graph
 *   brx_batch_config   the chosen shapes: locate threads, locate CTAs per
 *                      SM, q per tile, values and vectors smem budget (KB),
 *                      values and vectors CTAs per SM, number of tiles,
 *                      values and vectors gather warps per CTA of the
 *                      warp-independent FP32 gather (0: none), the least
 *                      element groups per mode (scalars + vectors) an item
 *                      needs to take that gather (-1: every item takes the
 *                      CTA-synchronous one), q per work descriptor of the
 *                      items below it (0: no such item) */
typedef struct brx_batch brx_batch;
brx_status brx_batch_create(brx_handle* const* handles, int32_t n, const int64_t* n_q, int32_t ir, uint32_t flags,
                            brx_batch** out);
void brx_batch_destroy(brx_batch* b);
brx_status brx_batch_set_io(brx_batch* b, const double* const* Q, void* const* values, void* const* vectors);
brx_status brx_batch_run(brx_batch* b, void* stream);
brx_status brx_batch_capture(brx_batch* b, void* stream);
brx_status brx_batch_launch(brx_batch* b, void* stream);
brx_status brx_batch_sync(brx_batch* b, void* stream, int32_t* failed);
brx_status brx_batch_tune(brx_batch* b, void* stream, int32_t reps);
brx_status brx_batch_config(const brx_batch* b, int32_t* cfg, int32_t n);
/* Set the shapes brx_batch_config reports (n ≥ 5: entries 0-4; entries 5-9
 * are derived and ignored; 10 and 11, when given, set the item split
 * between the two gathers and the small items' q per descriptor) and
 * re-plan; drops a captured graph. */
brx_status brx_batch_set_config(brx_batch* b, const int32_t* cfg, int32_t n);
int64_t brx_batch_launch_count(const brx_batch* b);
const char* brx_batch_last_error(const brx_batch* b);

/* Wait for work queued with BRX_FLAG_ASYNC (on `stream`, if given, and on
 * every stream that queued calls used) and report its status. */
brx_status brx_sync(brx_handle* h, void* stream);

/* Message for the last non-OK status on this handle (never NULL). */
const char* brx_last_error(const brx_handle* h);

/* Number of kernel launches this handle has issued since creation. */
int64_t brx_launch_count(const brx_handle* h);

/* Stage timing with CUDA events on the launching stream: enable (1) or
 * disable (0); either call clears the accumulated times. */
brx_status brx_profile(brx_handle* h, int32_t enable);

/* Milliseconds spent, since brx_profile, in the stages locate, grouping,
 * values gather and vectors gather (ms[0..3]), the q count they covered and
 * the number of gather work groups. */
brx_status brx_stage_times(const brx_handle* h, double* ms, int32_t n, int64_t* q_count, int64_t* groups);

/* Autotune the gathers of this handle on a sample query (Q: n × 3, host or
 * device; outputs as for brx_ir_interpolate_at, or NULL for temporary
 * device buffers; flags as for brx_ir_interpolate_at), timing with stage
 * events, best of reps: each gather's shared-memory budget per CTA (24-160
 * KB; it sets the modes staged per block and so the CTAs per SM), then,
 * for the heavier gather, the q per work descriptor (16-128) and the
 * work units per thread (1, 2, 4), and for FP32 data whether the
 * warp-independent gather (bulk-copied rows, per-warp mbarriers) or the
 * CTA-synchronous one is faster.  Results of FP64 data never change, those
 * of FP32 data only by rounding order.  brx_tuning returns values budget
 * (KB), vectors budget (KB), q per descriptor, units per thread, gather
 * kernel (0 warp-independent, 1 CTA-synchronous). */
brx_status brx_tune(brx_handle* h, const double* Q, int64_t n, void* values_out, void* vectors_out, uint32_t flags,
                    void* stream, int32_t reps);
brx_status brx_tuning(const brx_handle* h, int32_t* out, int32_t n);
/* Apply tuning values in brx_tuning's order (n ≥ 5), e.g. saved from an
 * earlier brx_tune; BRX_ERR_INVALID_ARGUMENT when one is out of range. */
brx_status brx_set_tuning(brx_handle* h, const int32_t* values, int32_t n);

int32_t brx_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BRX_H */
