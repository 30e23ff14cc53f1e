// Internal launch interface between the C ABI (api.cu) and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "device_math.cuh"

namespace fclg {

struct BatchArgs {
  const int4* shapes;     // fclg_shape[n_shapes]
  const float4* verts;    // xyzw
  const float4* pairs;    // fclg_pair[n_pairs]
  const float* guess;     // optional float[n_pairs][3]: GJKSolver::gjk_guess per pair
  const uint32_t* walk;   // optional [n_shapes]: first entry of each hull's walk block, or kNoWalk
  const float4* hull;     // walk blocks (hull.h), read by one-lane groups
  float4* results;        // fclg_result[n_pairs]
  uint32_t n_pairs;
  uint32_t n_shapes;
};

// Scratch of a query batch: the overlapping pairs handed from the GJK pass to
// the EPA pass.  count must be zero before the GJK pass.
struct EpaQueue {
  uint32_t* count;        // [1]
  uint32_t* list;         // [capacity] pair indices
  float4* rec;            // [capacity][7] final GJK simplex (rank, support points), which the EPA pass
                          // replaces by the entry's final-solve record; for the overflow list:
                          // [resume_cap] polytope states (kEpaResumeBytes each) or null
  uint32_t resume_cap = 0;  // overflow list: states the pool holds (the rest restart from the simplex)
  uint32_t* next = nullptr;  // zero before the EPA pass over this list: the count of entries its warps have
                             // taken (each warp takes its next entry there as it finishes one); null: each
                             // warp takes every (warps in the grid)-th entry
};
constexpr size_t kEpaRecordBytes = 7 * sizeof(float4);

// Separated pairs handed from the boolean GJK pass to the distance pass (the
// split one-lane launch, launch_gjk): each record is the pair, the separating
// vertex the distance loop starts from and the run it belongs to.  With a
// learned start, pairs whose distance from it is not certified go on to the
// redo list, which a third launch reruns from the plain direction.
struct DistList {
  uint32_t* count;       // [1] records written; zero before the boolean pass
  float4* rec;           // [capacity][3]: {pid, iterations of earlier runs, boolean iterations, stage},
                         // {pa.xyz, pb.x}, {pb.y, pb.z, 0, 0}; stage 0: plain run (the reference's stop),
                         // 1: learned start, 2: plain run with the certified stop
  uint32_t* next;        // [1] records taken by the distance pass; zero before it
  uint32_t* redo_count;  // [1] redo records written; zero before the boolean pass
  uint2* redo;           // [capacity] {pid, iterations of the learned-start run}
  uint32_t* redo_next;   // [1] redo records taken; zero before the redo pass
};
constexpr size_t kDistRecordBytes = 3 * sizeof(float4);
// Bytes of one small-layout polytope state handed to the large layout (epa.cuh EpaResume).
constexpr size_t kEpaResumeBytes = 6688;

// Scratch of the bucketing pass: pairs sorted by shape class (bucket.cu).
// box, sphere, capsule, cylinder, five bins of convex hulls up to big_nv vertices (by the
// power of two of the vertex count: < 16, < 32, < 64, < 128, more), convex > big_nv
constexpr int kHullBins = 5;
constexpr int kShapeClasses = 4 + kHullBins + 1;
constexpr int kBucketSmallKeys = kShapeClasses * kShapeClasses;
constexpr int kBucketKeys = 2 * kBucketSmallKeys;
static_assert(kBucketKeys <= 256, "bucket keys are bytes; the scan runs one thread per key");
struct BucketScratch {
  uint8_t* keys;      // [n] class key per pair
  uint32_t* order;    // [n] pair indices sorted by key
  uint32_t* hist;     // [kBucketKeys], zero between batches
  uint32_t* cursor;   // [kBucketKeys]
  uint32_t* ranges;   // [4]: [begin, end) of the small-pair launch, then of the large-pair launch
};

cudaError_t launch_bucketing(const BatchArgs& b, const BucketScratch& s, uint32_t big_nv, cudaStream_t st);

// GJK pass over order[range[0] .. range[1]) (order / range may be null: all
// pairs in index order) with `lanes` lanes per pair, as a persistent grid of
// `blocks` CTAs (0: one CTA per 128 lanes of work, not persistent).  refill:
// one-lane launches of queries without MPR or closed-form pairs run
// gjk_refill (lanes take new pairs as theirs finish) instead of gjk_pass<1>.
// next (optional, zero before the launch): the counter the persistent grid's
// warps take their pairs from.  dl (optional, capacity = the batch): where
// gjk_split_applies, the pass runs as two launches -- the boolean phase for
// every pair, which hands its separated pairs to dl, then the distance loop
// over dl -- so that no warp interleaves the two phases' code (same results).
cudaError_t launch_gjk(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, int lanes,
                       const uint32_t* order, const uint32_t* range, int blocks, cudaStream_t st,
                       bool refill = false, uint32_t* next = nullptr, const DistList* dl = nullptr);
// CTAs per SM the persistent GJK passes are compiled for (the default launch).
int gjk_default_ctas_per_sm();
// Whether launch_gjk with these arguments and a DistList runs the split launches
// (boolean, distance, and with a learned start the redo launch), and how many
// kernels that launch_gjk call then launches.
bool gjk_split_applies(const BatchArgs& b, const QueryParams& prm, int lanes, int blocks, bool refill);
int gjk_split_launches(const BatchArgs& b, const QueryParams& prm, int lanes, int blocks, bool refill);
// fcl::collide with directed penetration along b.guess (directed_pass.cu).
cudaError_t launch_directed(const BatchArgs& b, const QueryParams& prm, int blocks, cudaStream_t st);
// GJKSolver<double>::shapeDistance per pair in FP64, one thread per pair, as a
// grid of at most `blocks` CTAs of 128 (fp64_pass.cu); out = fclg_result64[n_pairs].
cudaError_t launch_gjk64(const BatchArgs& b, double tol, int max_iter, double* out, int blocks, cudaStream_t st);
cudaError_t prepare_epa();
// EPA over q's list: the small-polytope pass, then (when max_faces exceeds it)
// the large pass over the pairs ovf collected, then the final FP64 solves a
// thread per pair.  ovf.count must be zero and ovf.list hold q's capacity.
// q.rec's records are consumed (overwritten by the final-solve records).
cudaError_t launch_epa(const BatchArgs& b, const QueryParams& prm, const EpaQueue& q, const EpaQueue& ovf,
                       int num_sms, int ctas_per_sm, cudaStream_t st);
// Kernel launches launch_epa makes.
int epa_launches(const QueryParams& prm);
size_t epa_smem_bytes();
size_t epa_smem_bytes_large();
int epa_max_faces_supported();
// CTAs per SM the small-layout EPA kernel is compiled for (the default launch).
int epa_default_ctas_per_sm();

}  // namespace fclg
