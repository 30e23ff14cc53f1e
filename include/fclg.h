/*
 * fclg — batched narrowphase for one GB300 (sm_103a): the C ABI.
 *
 * Replaces, for batches of shape pairs, the reference's per-pair narrowphase
 * entry points (paths relative to the mind-fcl project root):
 *   fcl::collide(geom1, tf1, geom2, tf2, CollisionRequest, CollisionResult&)
 *       include/fcl/narrowphase/collision.h:54-58,
 *       include/fcl/narrowphase/collision_interface-inl.h:13-32
 *   detail::GJKSolver<S>::shapeSignedDistance / shapeIntersect
 *       include/fcl/narrowphase/detail/gjk_solver.h:53-177,
 *       include/fcl/narrowphase/detail/gjk_solver-inl.h:70-148, 810-874
 *   fcl::collide on two BVHModel<OBBRSS> (OrientedNodeBVHSolver::MeshIntersect)
 *       include/fcl/narrowphase/detail/traversal/collision/bvh_solver-inl.h:74-164
 *
 * Conventions
 *   - Plain pointers and sizes only.  Every function returns FCLG_OK (0) or a
 *     negative FCLG_E_* code; fclg_last_error() describes the last failure of
 *     a context.  A context is used by one host thread at a time.
 *   - Shape records follow the fcl geometry classes (Box stores full side
 *     lengths, Capsule / Cylinder radius and full length lz); type codes are
 *     the reference's GJKShapeType values (cvx_collide/gjk_shape.h:9-28).
 *   - A pair carries the pose of shape b expressed in shape a's frame
 *     (MinkowskiDiff::toshape0, gjk_solver-inl.h:84-85); every output point
 *     and normal is in shape a's frame.
 *   - Tolerances and limits default to what fcl::collide hands the solver
 *     (collision_request-inl.h:54-60, gjk_solver-inl.h:1120-1130).
 *   - *_device entry points take device pointers and a cudaStream_t (as
 *     void*) and are asynchronous; the others take host pointers and return
 *     when the results are in host memory.
 */
#ifndef FCLG_H_
#define FCLG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FCLG_OK = 0,
  FCLG_E_INVALID = -1,      /* bad argument (null pointer, index out of range, bad size) */
  FCLG_E_CUDA = -2,         /* a CUDA call failed; see fclg_last_error */
  FCLG_E_NO_SHAPES = -3,    /* query before fclg_set_shapes */
  FCLG_E_NO_DEVICE = -4,    /* no usable sm_103 device */
  FCLG_E_TOO_LARGE = -5     /* batch exceeds a fixed capacity */
};

/* GJKShapeType values, cvx_collide/gjk_shape.h:9-28 */
enum { FCLG_BOX = 0, FCLG_SPHERE = 1, FCLG_CAPSULE = 3, FCLG_CYLINDER = 5, FCLG_CONVEX = 100 };

typedef struct fclg_shape { /* 32 bytes */
  int32_t type;
  uint32_t vert_offset;  /* convex: first vertex in the vertex pool */
  uint32_t vert_count;   /* convex: number of hull vertices */
  uint32_t reserved;
  float param[4];        /* box: side x, y, z; sphere: radius; capsule, cylinder: radius, lz;
                            convex: interior point (vertex mean) x, y, z; [3]: bounding radius */
} fclg_shape;

typedef struct fclg_pair { /* 64 bytes */
  uint32_t shape_a, shape_b;
  float rot[9];          /* rotation of b's frame in a's frame, row-major */
  float trans[3];        /* origin of b in a's frame */
  uint32_t flags;        /* unused, 0 */
  uint32_t pair_class;   /* shape-pair class: the row of the warm-start model's embedding table
                            (fclg_warmstart_*); ignored without FCLG_REQ_WARM_START */
} fclg_pair;

typedef struct fclg_result { /* 48 bytes */
  float distance;        /* signed: separation > 0, -penetration depth < 0 */
  float normal[3];       /* unit; moving b along +normal increases the signed distance.  When
                            penetrating this is normalize(p_a - p_b), the reference's contact
                            normal (gjk_solver-inl.h:117-121) */
  float p_a[3];          /* witness point on a */
  float p_b[3];          /* witness point on b */
  int32_t status;        /* bits 0-7 GJK_Status (cvx_collide/gjk.h:13-28); bits 8-15 EPA_Status+1
                            (cvx_collide/epa.h:14), 0 when EPA did not run; bit 16
                            (FCLG_STATUS_MPR): a boolean decided by MPR */
  uint16_t iterations;   /* GJK (+distance) iterations, plus EPA expansions */
  uint8_t collide;       /* boolean collide flag */
  uint8_t ok;            /* the query produced a valid distance (shapeSignedDistance's return) */
} fclg_result;

typedef struct fclg_request {
  uint32_t gjk_max_iterations;  /* 0: 128 */
  uint32_t epa_max_faces;       /* 0: 256 (GJKSolver::epa_max_face_num) */
  uint32_t epa_max_iterations;  /* 0: 255 */
  uint32_t flags;               /* FCLG_REQ_* */
  float gjk_tolerance;          /* 0: 1e-6 (CollisionRequest::binaryCollisionTolerance) */
  float epa_tolerance;          /* 0: 1e-6 (CollisionRequest::distanceTolerance) */
  /* FCLG_REQ_WARM_START only.  A pair keeps the run from its learned
     direction only when that run certifies separation within warm_probe
     support evaluations (0: 3) and certifies its distance: the run's stop on a
     small improvement (gjk_distance.hpp:78-90) waits until the duality gap
     |v| - v^.w of its last support is at most warm_gap (0: 5e-6 m), so the
     distance is within warm_gap (plus FP32 rounding) of the exact one.  Every
     other pair (overlapping, probe exhausted, no certified distance) is redone
     from the plain direction under the same certified stop (overlapping pairs
     so get the plain GJK simplex and the plain EPA answer), and a pair that
     even then has no certified distance once more under the reference's own
     stop. */
  float warm_gap;
  uint32_t warm_probe;
} fclg_request;

enum {
  FCLG_REQ_BOOLEAN_ONLY = 1u << 0,  /* collide flag only: no distance, no EPA */
  FCLG_REQ_NO_EPA = 1u << 1,        /* separation distance only; overlapping pairs get distance 0 */
  FCLG_REQ_WARM_START = 1u << 2,    /* seed GJK with the learned direction model (fclg_warmstart_*) */
  FCLG_REQ_GJK_BOOLEAN = 1u << 3,   /* boolean collide by GJK instead of MPR (the reference's boolean
                                       fcl::collide runs MPR, falling back to GJK when MPR fails) */
  FCLG_REQ_NO_ANALYTIC = 1u << 4,   /* collide: sphere and box pairs by MPR / GJK+EPA instead of the
                                       closed-form solvers fcl::collide dispatches to (sphere-sphere,
                                       -capsule, -box, -cylinder, box-box; gjk_solver-inl.h:209-218) */
  FCLG_REQ_INCREMENTAL = 1u << 5    /* fclg_collide_directed*: the incremental minimum-distance
                                       penetration from the directions as hints instead of the
                                       directed penetration along them */
};
/* fclg_result.status bit 16: the boolean was decided by MPR.  Bit 17: the
   result came from a closed-form solver (sphere pairs, box-box: contact
   normal, the contact position +- depth / 2 along it as p_a / p_b; when
   apart, the centre-based separation (sphere pairs) or the gap along the
   separating axis found (box pairs) with p_a = p_b = 0). */
#define FCLG_STATUS_MPR (1 << 16)
#define FCLG_STATUS_ANALYTIC (1 << 17)

typedef struct fclg_context fclg_context;

/* Context on a device (sm_103 required).  Owns device copies of the shapes and
   the scratch of the query passes. */
int fclg_create(fclg_context** ctx, int device);
void fclg_destroy(fclg_context* ctx);
const char* fclg_last_error(const fclg_context* ctx);
/* Library version and the compute capability it was built for (e.g. 1030). */
int fclg_version(void);
int fclg_built_arch(void);

/* Shapes and hull vertices (float x, y, z, pad per vertex), copied to the
   device.  Replaces constructing fcl::Box / Sphere / Capsule / Cylinder /
   Convex objects (the geometry/shape headers). */
int fclg_set_shapes(fclg_context* ctx, const fclg_shape* shapes, uint32_t n_shapes, const float* vertices_xyzw,
                    uint64_t n_vertices);
/* Same, with the arrays already on the device; the context borrows them. */
int fclg_set_shapes_device(fclg_context* ctx, const fclg_shape* d_shapes, uint32_t n_shapes,
                           const float* d_vertices_xyzw, uint64_t n_vertices);

/* Broadphase over n posed objects -- object i is shape shape_ids[i] of
   fclg_set_shapes posed by poses[i] (world rotation row-major, translation:
   12 floats): every pair (i < j) whose world AABBs overlap (touching counts),
   the pair set BinaryAABB_Tree::SelfCollision reports
   (broadphase/binary_AABB_tree-inl.h) over CollisionObject::computeAABB's
   boxes (narrowphase/collision_object-inl.h:141-154: the local AABB
   translated for an identity rotation, else the cube of the local half
   diagonal about the moved centre).  pairs receives up to cap pairs (2 x
   u32, unordered); *n_pairs the total, which may exceed cap (call again with
   room for all).  aabbs (nullable, device entry: two float4 arrays lo / hi of
   n each; host entry: n x 6 floats lo, hi) receives the boxes.  The reference
   walks a binary tree; this sorts by the lower x bound and sweeps. */
int fclg_broadphase(fclg_context* ctx, const uint32_t* shape_ids, const float* poses, uint32_t n, uint32_t* pairs,
                    uint32_t cap, uint32_t* n_pairs, float* aabbs);
int fclg_broadphase_device(fclg_context* ctx, const uint32_t* d_shape_ids, const float* d_poses, uint32_t n,
                           uint32_t* d_pairs, uint32_t cap, uint32_t* d_n_pairs, float* d_aabb_lo, float* d_aabb_hi,
                           void* stream);
/* Two object sets (BinaryAABB_Tree::TreeCollision; a one-object set is
   SingleObjectCollision): every pair (i of the first set, j of the second)
   whose world AABBs overlap, as fclg_broadphase defines them; pairs hold
   (i, j) with i and j indices into their own sets.  Device pointers. */
int fclg_broadphase_cross_device(fclg_context* ctx, const uint32_t* d_shape_ids_a, const float* d_poses_a,
                                 uint32_t n_a, const uint32_t* d_shape_ids_b, const float* d_poses_b, uint32_t n_b,
                                 uint32_t* d_pairs, uint32_t cap, uint32_t* d_n_pairs, void* stream);
/* Narrowphase records (fclg_pair) for m candidate object pairs (2 x u32 each):
   shape_a = shape_ids[i], shape_b = shape_ids[j], the pose of j in i's frame
   (X_i^-1 X_j), flags and pair_class 0; feeds fclg_distance_device /
   fclg_collide_device straight from fclg_broadphase_device's output. */
int fclg_object_pairs_device(fclg_context* ctx, const uint32_t* d_shape_ids, const float* d_poses,
                             const uint32_t* d_candidates, uint32_t m, fclg_pair* d_pairs, void* stream);

/* Edge graph of the convex hull of nv points (xyzw), the graph the support
   walk climbs (fclg_tuning.support_walk): starts[6] = the extreme corner along
   +x, -x, +y, -y, +z, -z; first[nv + 1] = row starts into adj; adj = the
   neighbour corners of each vertex, rows ascending.  Points that are not
   corners of the hull get empty rows.  Host work only (no device, no context).
   Pass adj = NULL to learn *adj_len.  FCLG_E_INVALID when the points span no
   volume, FCLG_E_TOO_LARGE when adj_cap is short.  No counterpart in the
   reference's API: fcl::Convex derives the same graph from the face list its
   caller supplies (geometry/shape/convex-inl.h:379-405, FindVertexNeighbors). */
int fclg_hull_graph(const float* xyzw, uint32_t nv, uint32_t* starts, uint32_t* first, uint32_t* adj,
                    uint32_t adj_cap, uint32_t* adj_len);

/* Signed distance per pair: GJK separation distance and witness points for
   separated pairs, -EPA depth, witness points and contact normal for
   overlapping ones (GJKSolver::shapeSignedDistance, gjk_solver-inl.h:810-874;
   the reference exposes no fcl::distance for it).  req may be NULL. */
int fclg_distance(fclg_context* ctx, const fclg_pair* pairs, uint32_t n_pairs, const fclg_request* req,
                  fclg_result* results);
int fclg_distance_device(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const fclg_request* req,
                         fclg_result* d_results, void* stream);

/* Collision per pair (fcl::collide on a shape pair): the boolean flag, and with
   penetration (req NULL or without FCLG_REQ_BOOLEAN_ONLY) one contact per
   colliding pair — depth, normal, p_a / p_b — as useDefaultPenetration gives. */
int fclg_collide(fclg_context* ctx, const fclg_pair* pairs, uint32_t n_pairs, const fclg_request* req,
                 fclg_result* results);
int fclg_collide_device(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const fclg_request* req,
                        fclg_result* d_results, void* stream);

/* Separation distance in FP64 on the GPU: the GJK path of
   GJKSolver<double>::shapeDistance (ShapeDistanceIndepImpl,
   narrowphase/detail/gjk_solver-inl.h:760-798), one thread per pair running
   the reference's GJK boolean and GJK distance (cvx_collide/gjk.hpp:10-360,
   gjk_distance.hpp:10-559) in FP64, every operation rounded on its own in the
   reference's order, from the guess (1, 0, 0).  The FP32 inputs (shapes,
   vertices, poses) are taken exactly as FP64.  Every pair runs GJK: the
   closed-form specialisations shapeDistance has for sphere pairs and
   capsule-capsule (gjk_solver-inl.h:900-1000) are not taken.  A separated
   pair with valid witness points gets ok = 1, distance = |p_a - p_b| and the
   points (shape a's frame); every other pair gets ok = 0 and distance -1 (a
   separated pair whose witness extraction failed included: the reference
   returns its unset witness points there), collide = 1 when GJK reported an
   intersection.  req may be NULL (tolerance 1e-6, 128 iterations). */
typedef struct fclg_request64 {
  double gjk_tolerance;         /* 0: 1e-6 (GJKSolver::gjk_tolerance) */
  uint32_t gjk_max_iterations;  /* 0: 128 */
  uint32_t reserved;
} fclg_request64;
typedef struct fclg_result64 { /* 64 bytes */
  double distance;
  double p_a[3];
  double p_b[3];
  int32_t status;        /* GJK_Status (cvx_collide/gjk.h:13-28) */
  uint16_t iterations;   /* GJK boolean + distance iterations */
  uint8_t collide;
  uint8_t ok;
} fclg_result64;
int fclg_distance64(fclg_context* ctx, const fclg_pair* pairs, uint32_t n_pairs, const fclg_request64* req,
                    fclg_result64* results);
int fclg_distance64_device(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const fclg_request64* req,
                           fclg_result64* d_results, void* stream);

/* Signed distance on device pointers without any allocation in the call (no
   counterpart in the reference, whose per-pair solver keeps its polytope on
   the stack).  It runs the GJK pass unbucketed with the context's small-pair
   lane count: the same results as fclg_distance_device with bucketing off
   (fclg_tuning.bucketing = -1), and within the convex parity bar of the
   default bucketed launch.  The overlapping pairs handed from the GJK pass to
   the EPA pass are kept in a fixed device array of the library instead of
   context buffers, so n_pairs is at most FCLG_STATIC_MAX_PAIRS (larger
   batches return FCLG_E_TOO_LARGE; split them).  The first call on a device
   sets that array up (an address lookup, cached for the device's primary
   context; not valid across cudaDeviceReset): make it before any stream
   capture.  Calls on one device share the array, so calls that overlap in
   time on that device race; order them on one stream.  With profiling on,
   fclg_pass_times covers these calls too. */
#define FCLG_STATIC_MAX_PAIRS 16384u
int fclg_distance_device_static(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs,
                                const fclg_request* req, fclg_result* d_results, void* stream);

/* Learned warm start (no counterpart in the reference, whose GJKSolver takes
   one fixed or cached guess, gjk_solver-inl.h:1129).  A model predicts, per
   pair, the unit direction GJK starts from: an MLP over the relative pose
   (rot, trans) and a 16-float embedding of pair_class, three hidden layers of
   256 with GELU (tanh form), BF16 weights and FP32 accumulation on the tensor cores.
   Queries with FCLG_REQ_WARM_START on a context given a model by
   fclg_set_warmstart run GJK from that direction; a pair GJK finds
   overlapping, or that does not converge, is rerun from the plain direction,
   so EPA always starts from the plain simplex and the answer is the plain
   method's within its tolerance.  Parameters are FP32, in the order
   W1[256][32] b1[256] W2[256][256] b2 W3[256][256] b3 W4[8][256] b4[8]
   E[n_classes][16] (input columns: rot 0-8, trans 9-11, embedding 12-27,
   28-31 zero; rows 3-7 of W4 and b4 zero). */
typedef struct fclg_warmstart fclg_warmstart;
typedef struct fclg_train_config {
  uint32_t epochs;      /* 0: 1 */
  uint32_t batch;       /* multiple of 64; 0: 4096 */
  float lr;             /* Adam step at the start; 0: 1e-3 */
  float lr_final;       /* at the end (cosine decay); 0: lr / 20 */
  uint32_t seed;        /* shuffling */
  uint32_t reserved;
} fclg_train_config;
int fclg_warmstart_create(int device, uint32_t n_classes, uint32_t seed, fclg_warmstart** out);
void fclg_warmstart_destroy(fclg_warmstart* model);
const char* fclg_warmstart_last_error(const fclg_warmstart* model);
uint64_t fclg_warmstart_param_count(const fclg_warmstart* model);
int fclg_warmstart_get_params(const fclg_warmstart* model, float* params, uint64_t n_params);
int fclg_warmstart_set_params(fclg_warmstart* model, const float* params, uint64_t n_params);
/* Inference: d_out float[n][3], the unit direction (FCLG_WS_NORMALIZE) or the
   raw output y.  The queries use the tcgen05 kernel (TMEM accumulators,
   weights streamed by bulk async copies); FCLG_WS_MMA_SYNC selects the
   mma.sync kernel instead (the same model, for comparison). */
enum { FCLG_WS_NORMALIZE = 1u << 0, FCLG_WS_MMA_SYNC = 1u << 1 };
int fclg_warmstart_predict(fclg_warmstart* model, const fclg_pair* d_pairs, uint32_t n_pairs, float* d_out,
                           uint32_t flags, void* stream);
/* Synchronises the device; FCLG_E_CUDA if an inference launch since the last
   call gave up one of its bounded waits (the directions it owed are unset). */
int fclg_warmstart_status(fclg_warmstart* model);
/* The raw output y (float[n][3]) through the training kernels. */
int fclg_warmstart_forward(fclg_warmstart* model, const fclg_pair* d_pairs, uint32_t n_pairs, float* d_y,
                           void* stream);
/* Mean cosine loss 1 - <y/|y|, u> over n pairs (u: d_labels float[n][3],
   unit) and its gradient with respect to every parameter (host float[n_params]). */
int fclg_warmstart_gradient(fclg_warmstart* model, const fclg_pair* d_pairs, const float* d_labels, uint32_t n_pairs,
                            float* grad, float* loss);
/* Adam on shuffled mini-batches; epoch_loss (host, nullable) receives the mean
   loss of each epoch.  Synchronous. */
int fclg_warmstart_train(fclg_warmstart* model, const fclg_pair* d_pairs, const float* d_labels, uint32_t n_pairs,
                         const fclg_train_config* config, float* epoch_loss);
/* Model used by queries that set FCLG_REQ_WARM_START (NULL: none; such queries
   then fail).  The model must outlive its use by the context. */
int fclg_set_warmstart(fclg_context* ctx, fclg_warmstart* model);

/* fcl::collide with CollisionRequest::useDirectedPenetration
   (collisionPenetrationMPR, collision_penetration-inl.h:106-250): the boolean
   collide (closed form for sphere pairs, MPR with the GJK fallback otherwise),
   then for colliding pairs MPR::RunDirectedPenetration (cvx_collide/mpr.hpp:
   495-701) along dirs[i] (float[n][3], unit: shape b's escape direction in
   shape a's frame).  Per pair: collide; distance = -(depth along the
   direction) and ok = 1 when the directed run succeeded; normal = the
   direction; p_a / p_b the directed witness points; status bit 18
   (FCLG_STATUS_DIRECTED) with the directed status + 1 in bits 8-15 (0 OK,
   1 Failed, 2 FailedNoIntersect, 3 iteration limit).
   With FCLG_REQ_INCREMENTAL in req->flags: CollisionRequest::
   useIncrementalMinimumDistancePenetration instead -- for colliding pairs
   MPR::IncrementalMinimumPenetrationDistance (cvx_collide/
   mpr_incremental_penetration.hpp:10-333, 128 iterations, returning on the
   first converged direction) from dirs[i] as the hint.  Per pair: distance =
   -depth and ok = 1 when the run is OK or stopped at its iteration limit
   (both valid penetrations for the reference); normal = the direction it
   settled on (the hint when not ok); status bit 19 (FCLG_STATUS_INCREMENTAL)
   with the incremental status + 1 in bits 8-15 (0 OK, 1 Failed,
   2 FailedNoIntersect, 4 iteration limit).
   With FCLG_REQ_INCREMENTAL | FCLG_REQ_WARM_START the hints are the unit
   directions of the context's warm-start model (fclg_set_warmstart; dirs may
   be NULL), so for this use it is trained on penetrating pairs' result
   normals (shape b's escape direction).  FCLG_REQ_WARM_START without
   FCLG_REQ_INCREMENTAL, or without a model, is FCLG_E_INVALID. */
#define FCLG_STATUS_DIRECTED (1 << 18)
#define FCLG_STATUS_INCREMENTAL (1 << 19)
int fclg_collide_directed(fclg_context* ctx, const fclg_pair* pairs, uint32_t n_pairs, const float* dirs,
                          const fclg_request* req, fclg_result* results);
int fclg_collide_directed_device(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const float* d_dirs,
                                 const fclg_request* req, fclg_result* d_results, void* stream);

/* Launch shape of the query passes.  Pairs are first sorted on the device by
   shape class (box / sphere / capsule / cylinder / convex hull, hulls split at
   large_hull_vertices); pairs without a large hull run the GJK pass with
   gjk_lanes_small lanes per pair, the rest with gjk_lanes_large.  Zero
   fields keep the current value.  Defaults: bucketing on, 1 and 4 lanes,
   128 vertices, 4 GJK and 6 EPA CTAs per SM (the EPA pass's first,
   128-face layout), support walk off, GJK refill off.
   gjk_refill: one-lane GJK launches of distance queries, warm-started or not
   (and of collides without MPR or closed-form pairs) keep every lane of a warp busy by handing
   a lane whose pair has finished the next pair of its warp's share, instead
   of letting 32 pairs wait for the slowest of them; answers are the same.
   On GB300 it pays where supports are costly (hulls of 64-256 vertices:
   6 % faster) and costs where they are cheap (4-15 % slower); fclg_autotune
   tries both.
   support_walk: hulls of more than 32 vertices get their edge graph built on
   the host when shapes are set (a quickhull per hull, spread over the host's
   threads); a GJK / MPR launch with one lane per pair then finds a hull's
   support by hill-climbing that graph from one of six cached axis-extreme
   corners, the rule of Convex::findExtremeVertexViaNeighbours
   (geometry/shape/convex-inl.h:201-283), instead of scanning every vertex.
   Groups of several lanes and the EPA pass scan.  Both give the vertex of
   maximal support value; they may differ only where several vertices tie.
   Off by default: on GB300 the one-lane scan of an L1-resident hull measured
   faster (lanes of a warp walk paths of different lengths); fclg_autotune
   tries both. */
typedef struct fclg_tuning {
  int32_t bucketing;            /* 1 on, -1 off, 0 unchanged */
  int32_t gjk_lanes_small;      /* 1, 2, 4, 8, 16 or 32 */
  int32_t gjk_lanes_large;
  int32_t large_hull_vertices;
  int32_t gjk_ctas_per_sm;
  int32_t epa_ctas_per_sm;      /* small-layout EPA CTAs per SM (two 13-warp CTAs by default) */
  int32_t support_walk;         /* 1 on, -1 off, 0 unchanged */
  int32_t gjk_refill;           /* 1 on, -1 off, 0 unchanged */
  int32_t epa_resume;           /* 1 on (default), -1 off, 0 unchanged: a pair whose EPA polytope
                                   outgrows the 128-face layout continues in the 256-face layout
                                   from where it stopped instead of starting over (same answers) */
} fclg_tuning;
int fclg_set_tuning(fclg_context* ctx, const fclg_tuning* tuning);
int fclg_get_tuning(const fclg_context* ctx, fclg_tuning* tuning);
/* Shorthand: the same lane count for both GJK launches, and the EPA CTAs per SM. */
int fclg_set_launch(fclg_context* ctx, int gjk_lanes, int epa_ctas_per_sm);

/* Autotuner: times the query on (d_pairs, n) under each candidate launch shape
   (GJK lanes for small / large hulls: 1-8 / 4-16, hull split 64 / 128 / 256
   vertices, bucketing on / off; three queries each), keeps the fastest on the
   context and returns it with its time per query.  d_results is overwritten.
   No counterpart in the reference. */
int fclg_autotune(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const fclg_request* req,
                  fclg_result* d_results, int distance_query, fclg_tuning* best, float* best_ms);

/* CUDA graph of one whole query (bucketing, both GJK launches, EPA, and the
   warm-start inference when requested) on fixed device buffers: capture once,
   then replay with fclg_graph_launch after refilling d_pairs.  The capture
   allocates the query's scratch first; a graph goes stale (launch returns
   FCLG_E_INVALID) when the context later reallocates that scratch for a
   larger batch or its shapes are set again.  No counterpart in the reference. */
typedef struct fclg_graph fclg_graph;
int fclg_graph_create(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs, const fclg_request* req,
                      fclg_result* d_results, int distance_query, fclg_graph** graph);
int fclg_graph_launch(fclg_context* ctx, fclg_graph* graph, void* stream);
void fclg_graph_destroy(fclg_graph* graph);

/* Kernel launches issued by this context since creation (for accounting). */
uint64_t fclg_launch_count(const fclg_context* ctx);

/* Per-pass timing: when enabled, every query records CUDA events around its
   GJK and EPA passes on the query's stream; fclg_pass_times synchronises on
   them and returns the summed milliseconds of each pass and the number of
   queries timed since the last reset (reset = 1 clears the sums). */
int fclg_set_profiling(fclg_context* ctx, int enable);
int fclg_pass_times(fclg_context* ctx, double* gjk_ms, double* epa_ms, uint64_t* queries, int reset);

/* ---------------------------------------------------------------- meshes --
   Triangle meshes with an OBB bounding-volume hierarchy built on the host
   (replaces BVHModel<OBBRSS>::beginModel / addSubModel / endModel,
   geometry/bvh/BVH_model-inl.h:136-303), and batched boolean mesh-mesh
   collision (fcl::collide on two BVHModel<OBBRSS> with penetration off:
   OrientedNodeBVHSolver::MeshIntersect, bvh_solver-inl.h:74-164). */
typedef struct fclg_mesh fclg_mesh;

typedef struct fclg_mesh_node { /* 64 bytes */
  float axis[9];    /* row-major; the columns are the box axes */
  float center[3];
  float extent[3];  /* half sizes */
  int32_t child;    /* >= 0: children child and child + 1; < 0: leaf of triangle -(child + 1) */
} fclg_mesh_node;

/* Builds the hierarchy on the host only (no device, no context): 2 x
   n_triangles - 1 nodes, root first, and the triangle soup
   (n_triangles x 3 x xyzw floats).  The tree is the reference's own
   (BVHModel<OBBRSS<double>>::endModel with the default mean splitter: same
   node slots, children and leaf triangles, built in FP64 from the FP32
   vertices); each stored FP32 box contains its triangles.  Returns FCLG_OK or
   FCLG_E_INVALID. */
int fclg_bvh_build(const float* vertices_xyz, uint32_t n_vertices, const int32_t* triangles, uint32_t n_triangles,
                   fclg_mesh_node* nodes, float* triangles_xyzw);

/* The FP64 |extent|^2 of each node's box as the reference's
   BVHModel<OBBRSS<double>> computes it (OBB::size, math/bv/OBB-inl.h:153-156;
   the mesh traversal descends into the pair's node with the larger value,
   bvh_solver-inl.h:150-151) and the tree's depth (deepest level, root 0), on
   the host only.  sizes (nullable) holds 2 x n_triangles - 1 values.  Returns
   FCLG_OK or FCLG_E_INVALID. */
int fclg_bvh_node_sizes(const float* vertices_xyz, uint32_t n_vertices, const int32_t* triangles,
                        uint32_t n_triangles, double* sizes, uint32_t* depth);

/* Builds the hierarchy over triangles (3 vertex indices each) and uploads
   it to the context's device. */
int fclg_mesh_create(fclg_context* ctx, const float* vertices_xyz, uint32_t n_vertices, const int32_t* triangles,
                     uint32_t n_triangles, fclg_mesh** mesh);
void fclg_mesh_destroy(fclg_mesh* mesh);
int fclg_mesh_info(const fclg_mesh* mesh, uint32_t* n_nodes, uint32_t* n_triangles);
/* Copies the flattened hierarchy (n_nodes nodes) and the triangle soup
   (n_triangles x 3 x xyzw floats) to host memory. */
int fclg_mesh_export(const fclg_mesh* mesh, fclg_mesh_node* nodes, float* triangles_xyzw);

/* Boolean collision of mesh b posed by poses[i] (rotation row-major, then
   translation: 12 floats, b in a's frame) against mesh a.  A pose stops after
   max_contacts colliding triangle pairs (CollisionRequest::num_max_contacts;
   1 is first-contact mode): the first max_contacts in the reference's own
   traversal order, listed in that order, i.e. the reference's contact list.
   Outputs per pose: flags (1 if colliding), counts, pairs (max_contacts x 2
   triangle ids of a and b) and, when not NULL, status (bit 0: the traversal
   stack overflowed, the pair set may be incomplete; bit 1: round limit).
   FCLG_E_TOO_LARGE when the two trees' depths sum above 62 (the traversal
   orders node pairs by a 64-bit path key). */
int fclg_mesh_collide(fclg_context* ctx, const fclg_mesh* a, const fclg_mesh* b, const float* poses, uint32_t n_poses,
                      uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* pairs, uint32_t* status);
int fclg_mesh_collide_device(fclg_context* ctx, const fclg_mesh* a, const fclg_mesh* b, const float* d_poses,
                             uint32_t n_poses, uint32_t max_contacts, uint8_t* d_flags, uint32_t* d_counts,
                             int32_t* d_pairs, uint32_t* d_status, void* stream);
/* Work of the mesh-mesh queries run while profiling is on
   (fclg_set_profiling): node pairs whose boxes were tested and triangle pairs
   tested, summed since the last reset (reset = 1 clears them); the inputs of
   the traversal's bytes (64 B per node read, 48 B per triangle read).
   Synchronises the device.  No counterpart in the reference. */
int fclg_mesh_traffic(fclg_context* ctx, uint64_t* node_pairs, uint64_t* triangle_pairs, int reset);

/* Boolean collision of a mesh against shapes of the context (fcl::collide on
   a BVHModel<OBBRSS> and a shape with penetration off:
   OrientedNodeBVHSolver::MeshShapeIntersect, bvh_solver-inl.h:6-72, with the
   shape-triangle tests GJKSolver::shapeTriangleIntersect picks,
   gjk_solver-inl.h:451-591: sphere-triangle and box-triangle in closed form,
   MPR for capsules, cylinders and hulls).  Query i: shape shape_ids[i] (of
   fclg_set_shapes) posed by poses[i] (rotation row-major, then translation:
   12 floats) in the mesh's frame.  A query stops after max_contacts colliding
   triangles (1: first-contact mode).  Outputs per query: flags, counts,
   tri_ids (max_contacts triangle ids) and, when not NULL, status (bit 0 stack
   overflow, bit 1 round limit, bit 2 shape id out of range). */
int fclg_mesh_shape_collide(fclg_context* ctx, const fclg_mesh* mesh, const uint32_t* shape_ids, const float* poses,
                            uint32_t n, uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* tri_ids,
                            uint32_t* status);
int fclg_mesh_shape_collide_device(fclg_context* ctx, const fclg_mesh* mesh, const uint32_t* d_shape_ids,
                                   const float* d_poses, uint32_t n, uint32_t max_contacts, uint8_t* d_flags,
                                   uint32_t* d_counts, int32_t* d_tri_ids, uint32_t* d_status, void* stream);

/* The same with penetration on (a CollisionRequest with contacts,
   ShapePairIntersectSolver::ShapeSimplexIntersect, narrowphase/detail/
   shape_pair_intersect-inl.h:132-170): leaves other than spheres decide by
   GJK, and every reported triangle gets its contact in contacts[n][max_contacts]
   [8]: pos (3, mesh frame), normal (3, reversed as the reference's mesh-shape
   contact meta does, bvh_solver-inl.h:56-61), penetration depth, and status
   bits as a float's bits (0-7: EPA status + 1, 0 for the closed-form sphere;
   bit 8: GJK or EPA gave no contact, which the reference would not have
   added).  Sphere leaves are sphereTriangleIntersect's contact (its depth is
   -(r - distance), as the reference writes it). */
int fclg_mesh_shape_contacts(fclg_context* ctx, const fclg_mesh* mesh, const uint32_t* shape_ids, const float* poses,
                             uint32_t n, uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* tri_ids,
                             float* contacts, uint32_t* status);
int fclg_mesh_shape_contacts_device(fclg_context* ctx, const fclg_mesh* mesh, const uint32_t* d_shape_ids,
                                    const float* d_poses, uint32_t n, uint32_t max_contacts, uint8_t* d_flags,
                                    uint32_t* d_counts, int32_t* d_tri_ids, float* d_contacts, uint32_t* d_status,
                                    void* stream);

/* ---- translational continuous collision --------------------------------
   Replaces fcl::translational_ccd(o1, tf1, o1_displacement, o2, tf2, request,
   result) (narrowphase/continuous_collision.h:13-19) on shape pairs, through
   ShapePairTranslationalCollisionSolver::RunShapePair
   (narrowphase/detail/ccd/shape_pair_ccd-inl.h:113-160).  Per pair, shape a
   moves from the pair's start along disp[i].axis (unit, shape a's frame; the
   TranslationalDisplacement of ccd_typedef.h:11-15) by disp[i].distance
   (>= 0); shape b stays at the pair's pose.  Box-box pairs always take the
   box interval test (BoxPairTranslationalCCD::IsDisjoint); the other pairs
   the swept-volume MPR, after that test on the shapes' local boxes for
   FCLG_TOC_BOX. */
typedef struct {
  float axis[3];
  float distance;
} fclg_displacement;

enum {  /* TimeOfCollisionRequestType (narrowphase/detail/ccd/ccd_request.h:11-17) */
  FCLG_TOC_NONE = 0,    /* kNotRequested: the boolean alone (box-box pairs still report their interval) */
  FCLG_TOC_BOX = 1,     /* kBoxApproximate: the local boxes' interval, then MPR */
  FCLG_TOC_SAMPLE = 2   /* kOneTocSample: one time of collision from MPR's final portal */
};

typedef struct {            /* ContinuousCollisionRequest (ccd_request.h:19-31); 0 = default */
  uint32_t toc_type;        /* FCLG_TOC_* */
  int32_t max_gjk_iterations;       /* 128 */
  float gjk_tolerance;              /* 1e-6 */
  uint32_t reserved;
  double zero_movement_tolerance;   /* 1e-4 */
} fclg_ccd_request;

typedef struct {     /* one ContinuousCollisionContact's verdict (ccd_contact.h) */
  uint32_t collide;  /* 1: the moving shape touches the other somewhere on its path */
  uint32_t status;   /* bits 0-1 swept MPR status (0 Intersect, 1 Separated, 2 Failed, 3 not run),
                        bit 2 box interval test ran, bit 3 it found the boxes disjoint,
                        bit 4 shape id out of range */
  float toc_lower;   /* time of collision in [0, 1] as a fraction of the distance: */
  float toc_upper;   /* the box interval, the one sample (lower = upper), or -1 when none */
} fclg_ccd_result;

int fclg_translational_ccd(fclg_context* ctx, const fclg_pair* pairs, uint32_t n_pairs, const fclg_displacement* disp,
                           const fclg_ccd_request* req, fclg_ccd_result* results);
int fclg_translational_ccd_device(fclg_context* ctx, const fclg_pair* d_pairs, uint32_t n_pairs,
                                  const fclg_displacement* d_disp, const fclg_ccd_request* req,
                                  fclg_ccd_result* d_results, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FCLG_H_ */
