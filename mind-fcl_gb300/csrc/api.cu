// The C ABI of include/fclg.h: contexts, shape upload, and the batched
// collide / distance queries over the GJK and EPA passes (gjk_pass*.cu, epa_pass.cu).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <atomic>
#include <thread>

#include "broadphase.h"
#include "fclg.h"
#include "hull.h"
#include "ccd.h"
#include "kernels.h"
#include "mesh_build.h"
#include "mesh_kernels.h"
#include "warmstart.h"

// Counters of a query (fclg_context::epa_count): EPA work list and overflow
// list lengths, entries taken by the two EPA launches and by the two GJK
// launches, then the separated-pair list's and the redo list's lengths and
// entries taken.
constexpr int kQueueCounters = 10;

struct fclg_context {
  int device = 0;
  int num_sms = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  // shapes
  void* own_shapes = nullptr;
  void* own_verts = nullptr;
  const int4* shapes = nullptr;
  const float4* verts = nullptr;
  uint32_t n_shapes = 0;
  uint64_t n_verts = 0;
  // support walk: per-shape first entry of the hull's walk block (or kNoWalk), the blocks
  uint32_t* walk_tab = nullptr;
  float4* hull_ents = nullptr;
  uint32_t walk_hulls = 0;
  bool support_walk = false;
  // broadphase scratch and host staging
  void* bp_scratch = nullptr;
  size_t bp_bytes = 0;
  void* bp_io = nullptr;
  size_t bp_io_bytes = 0;
  void* bp_join = nullptr;  // the two sets of a cross query, side by side
  size_t bp_join_bytes = 0;
  bool gjk_refill = false;
  // scratch handed from the GJK pass to the EPA pass
  uint32_t* epa_count = nullptr;  // [kQueueCounters]
  uint32_t* epa_list = nullptr;
  uint32_t* epa_ovf = nullptr;
  unsigned char* epa_resume = nullptr;  // polytope states handed from the small EPA layout to the large one
  uint32_t epa_resume_cap = 0;
  bool epa_resume_on = true;
  float4* epa_rec = nullptr;
  size_t epa_cap = 0;
  // device staging of the host-pointer entry points
  void* io_pairs = nullptr;
  void* io_results = nullptr;
  size_t io_cap = 0;
  // bucketing scratch
  uint8_t* bk_keys = nullptr;
  uint32_t* bk_order = nullptr;
  uint32_t* bk_small = nullptr;  // hist | cursor | ranges
  float4* bk_dist = nullptr;     // separated pairs between the split GJK launches (fclg::DistList)
  uint2* bk_redo = nullptr;      // learned-start pairs rerun from the plain direction (fclg::DistList)
  size_t bk_cap = 0;
  // launch shape
  bool bucketing = true;
  int gjk_lanes = 1;
  int gjk_lanes_large = 4;
  int large_hull = 128;
  int gjk_ctas_per_sm = fclg::gjk_default_ctas_per_sm();
  int epa_ctas_per_sm = fclg::epa_default_ctas_per_sm();
  uint64_t launches = 0;
  // optional per-pass timing
  bool profiling = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  bool ev_pending = false;
  bool ev_epa = false;
  double gjk_ms = 0, epa_ms = 0;
  uint64_t timed = 0;
  // device staging of the host-pointer mesh entry point
  void* mesh_io = nullptr;
  size_t mesh_io_bytes = 0;
  // per-warp contact buffers of mesh-mesh requests above the shared-memory buffer
  void* mesh_cbuf = nullptr;
  size_t mesh_cbuf_bytes = 0;
  // mesh-mesh traffic counters while profiling: node pairs and triangle pairs tested
  unsigned long long* mesh_ctr = nullptr;
  uint32_t* mesh_take = nullptr;  // work taken by a persistent launch's warps (mesh, mesh-shape, CCD)
  uint32_t* contact_take = nullptr;  // contact slots taken by the mesh-shape contact launch's warps
  // learned warm start: the model and its per-pair directions
  fclg_warmstart* ws = nullptr;
  float* guess = nullptr;
  size_t guess_cap = 0;
  // bumped whenever query scratch is reallocated (invalidates captured graphs)
  uint64_t scratch_epoch = 0;
  // translational CCD: hull boxes of the current shapes (2 float4 each), host staging of displacements
  float4* hull_aabb = nullptr;
  bool hull_aabb_valid = false;
  void* ccd_disp = nullptr;
  size_t ccd_disp_cap = 0;
};

struct fclg_mesh {
  int device = 0;
  void* nodes = nullptr;
  void* tris = nullptr;
  void* sizes = nullptr;  // FP64 |extent|^2 per node (the traversal's descend key)
  uint32_t n_nodes = 0;
  uint32_t n_tris = 0;
  uint32_t depth = 0;     // deepest node level (root 0)
};

namespace {

int fail(fclg_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// The CUDA runtime is shared with the rest of the process (PyTorch, the
// caller): a non-sticky error some other caller left pending would otherwise
// be reported by this library's first launch check.  Entry points that launch
// clear it first; sticky errors (a faulted context) cannot be cleared and are
// still reported by the calls that follow.
inline void clear_pending_error() {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess && getenv("FCLG_DEBUG_PENDING"))
    fprintf(stderr, "fclg: cleared a pending CUDA error at entry: %s\n", cudaGetErrorString(e));
}

int cuda_fail(fclg_context* c, cudaError_t e, const char* what) {
  return fail(c, FCLG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define FCLG_CUDA(ctx, call)                                   \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);   \
  } while (0)

int validate_shapes(fclg_context* c, const fclg_shape* s, uint32_t n, uint64_t n_verts) {
  for (uint32_t i = 0; i < n; ++i) {
    const int t = s[i].type;
    if (t == FCLG_CONVEX) {
      if (s[i].vert_count == 0 || (uint64_t)s[i].vert_offset + s[i].vert_count > n_verts) {
        char b[160];
        snprintf(b, sizeof b, "shape %u: convex vertex range [%u, +%u) outside the %llu-vertex pool", i,
                 s[i].vert_offset, s[i].vert_count, (unsigned long long)n_verts);
        return fail(c, FCLG_E_INVALID, b);
      }
    } else if (t != FCLG_BOX && t != FCLG_SPHERE && t != FCLG_CAPSULE && t != FCLG_CYLINDER) {
      char b[96];
      snprintf(b, sizeof b, "shape %u: unsupported type %d", i, t);
      return fail(c, FCLG_E_INVALID, b);
    }
  }
  return FCLG_OK;
}

void release_shapes(fclg_context* c) {
  if (c->own_shapes) cudaFree(c->own_shapes);
  if (c->own_verts) cudaFree(c->own_verts);
  if (c->walk_tab) cudaFree(c->walk_tab);
  if (c->hull_ents) cudaFree(c->hull_ents);
  c->walk_tab = nullptr;
  c->hull_ents = nullptr;
  c->walk_hulls = 0;
  if (c->hull_aabb) cudaFree(c->hull_aabb);
  c->hull_aabb = nullptr;
  c->hull_aabb_valid = false;
  c->scratch_epoch += 1;  // captured graphs hold the old shape pointers
  c->own_shapes = c->own_verts = nullptr;
  c->shapes = nullptr;
  c->verts = nullptr;
  c->n_shapes = 0;
  c->n_verts = 0;
}

// Walk blocks of every hull above kWalkMinVertices (hull.h), built in
// parallel over distinct vertex ranges and uploaded with a per-shape table.
// A hull whose points span no volume, or whose graph does not fit a block,
// keeps the vertex scan.
int build_walks(fclg_context* c, const fclg_shape* s, uint32_t n, const float* verts) {
  std::vector<uint32_t> tab(n, fclg::kNoWalk);
  std::vector<uint64_t> keys;
  for (uint32_t i = 0; i < n; ++i)
    if (s[i].type == FCLG_CONVEX && s[i].vert_count > fclg::kWalkMinVertices)
      keys.push_back(((uint64_t)s[i].vert_offset << 32) | s[i].vert_count);
  if (keys.empty()) return FCLG_OK;
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<std::vector<float>> blocks(keys.size());
  std::atomic<size_t> next{0};
  auto work = [&]() {
    fclg::HullGraph g;
    for (size_t k = next.fetch_add(1); k < keys.size(); k = next.fetch_add(1)) {
      const float* v = verts + 4 * (size_t)(keys[k] >> 32);
      const uint32_t nv = (uint32_t)keys[k];
      if (!fclg::hull_graph(v, nv, g) || !fclg::pack_walk(v, g, blocks[k])) blocks[k].clear();
    }
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>({(size_t)hw, (size_t)64, keys.size() / 8 + 1});
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  std::vector<uint32_t> base(keys.size(), fclg::kNoWalk);
  uint64_t total = 0;
  uint32_t built = 0;
  for (size_t k = 0; k < keys.size(); ++k) {
    const uint64_t ents = blocks[k].size() / 4;
    if (ents == 0 || total + ents >= fclg::kNoWalk) continue;
    base[k] = (uint32_t)total;
    total += ents;
    ++built;
  }
  if (total == 0) return FCLG_OK;
  for (uint32_t i = 0; i < n; ++i) {
    if (s[i].type != FCLG_CONVEX || s[i].vert_count <= fclg::kWalkMinVertices) continue;
    const uint64_t key = ((uint64_t)s[i].vert_offset << 32) | s[i].vert_count;
    tab[i] = base[std::lower_bound(keys.begin(), keys.end(), key) - keys.begin()];
  }
  std::vector<float> ents;
  ents.reserve(4 * total);
  for (size_t k = 0; k < keys.size(); ++k)
    if (base[k] != fclg::kNoWalk) ents.insert(ents.end(), blocks[k].begin(), blocks[k].end());
  FCLG_CUDA(c, cudaMalloc(&c->walk_tab, (size_t)n * sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMalloc(&c->hull_ents, total * sizeof(float4)));
  FCLG_CUDA(c, cudaMemcpy(c->walk_tab, tab.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  FCLG_CUDA(c, cudaMemcpy(c->hull_ents, ents.data(), total * sizeof(float4), cudaMemcpyHostToDevice));
  c->walk_hulls = built;
  return FCLG_OK;
}

// Batch arguments over the context's shapes.
fclg::BatchArgs batch_args(const fclg_context* c) {
  fclg::BatchArgs b{};
  b.shapes = c->shapes;
  b.verts = c->verts;
  b.walk = c->support_walk ? c->walk_tab : nullptr;
  b.hull = c->hull_ents;
  b.n_shapes = c->n_shapes;
  return b;
}

int ensure_epa(fclg_context* c, size_t n) {
  if (n <= c->epa_cap) return FCLG_OK;
  if (c->epa_list) cudaFree(c->epa_list);
  if (c->epa_ovf) cudaFree(c->epa_ovf);
  if (c->epa_rec) cudaFree(c->epa_rec);
  if (c->epa_resume) cudaFree(c->epa_resume);
  c->epa_list = nullptr;
  c->epa_ovf = nullptr;
  c->epa_rec = nullptr;
  c->epa_resume = nullptr;
  c->epa_resume_cap = 0;
  c->epa_cap = 0;
  c->scratch_epoch += 1;  // captured graphs hold the freed buffers, also if the allocation below fails
  const size_t cap = std::max<size_t>(n, 1024);
  FCLG_CUDA(c, cudaMalloc(&c->epa_list, cap * sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMalloc(&c->epa_ovf, cap * sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMalloc(&c->epa_rec, cap * fclg::kEpaRecordBytes));
  // states of the pairs that outgrow the small EPA layout (a few per cent of
  // the overlapping pairs); pairs past the pool rerun from their simplex
  const size_t resume_cap = std::min<size_t>(std::max<size_t>(cap / 16, 1024), 262144);
  FCLG_CUDA(c, cudaMalloc(&c->epa_resume, resume_cap * fclg::kEpaResumeBytes));
  c->epa_resume_cap = (uint32_t)resume_cap;
  c->epa_cap = cap;
  return FCLG_OK;
}

int ensure_bucket(fclg_context* c, size_t n) {
  if (!c->bk_small) {
    FCLG_CUDA(c, cudaMalloc(&c->bk_small, (2 * fclg::kBucketKeys + 4) * sizeof(uint32_t)));
    FCLG_CUDA(c, cudaMemset(c->bk_small, 0, (2 * fclg::kBucketKeys + 4) * sizeof(uint32_t)));
  }
  if (n <= c->bk_cap) return FCLG_OK;
  if (c->bk_keys) cudaFree(c->bk_keys);
  if (c->bk_order) cudaFree(c->bk_order);
  if (c->bk_dist) cudaFree(c->bk_dist);
  if (c->bk_redo) cudaFree(c->bk_redo);
  c->bk_keys = nullptr;
  c->bk_order = nullptr;
  c->bk_dist = nullptr;
  c->bk_redo = nullptr;
  c->bk_cap = 0;
  c->scratch_epoch += 1;
  const size_t cap = std::max<size_t>(n, 1024);
  FCLG_CUDA(c, cudaMalloc(&c->bk_keys, cap));
  FCLG_CUDA(c, cudaMalloc(&c->bk_order, cap * sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMalloc(&c->bk_dist, cap * fclg::kDistRecordBytes));
  FCLG_CUDA(c, cudaMalloc(&c->bk_redo, cap * sizeof(uint2)));
  c->bk_cap = cap;
  return FCLG_OK;
}

int ensure_io(fclg_context* c, size_t n) {
  if (n <= c->io_cap) return FCLG_OK;
  if (c->io_pairs) cudaFree(c->io_pairs);
  if (c->io_results) cudaFree(c->io_results);
  c->io_pairs = c->io_results = nullptr;
  c->io_cap = 0;
  const size_t cap = std::max<size_t>(n, 1024);
  FCLG_CUDA(c, cudaMalloc(&c->io_pairs, cap * sizeof(fclg_pair)));
  FCLG_CUDA(c, cudaMalloc(&c->io_results, cap * sizeof(fclg_result)));
  c->io_cap = cap;
  return FCLG_OK;
}

int ensure_guess(fclg_context* c, size_t n) {
  if (n <= c->guess_cap) return FCLG_OK;
  if (c->guess) cudaFree(c->guess);
  c->guess = nullptr;
  c->guess_cap = 0;
  c->scratch_epoch += 1;
  const size_t cap = std::max<size_t>(n, 1024);
  FCLG_CUDA(c, cudaMalloc(&c->guess, cap * 3 * sizeof(float)));
  c->guess_cap = cap;
  return FCLG_OK;
}

// Defaults of fclg_request.warm_probe / warm_gap.
constexpr int kWarmProbeDefault = 3;
constexpr float kWarmGapDefault = 5e-6f;

fclg::QueryParams make_params(const fclg_request* req, bool distance_query) {
  fclg::QueryParams p;
  p.gjk_tol = (req && req->gjk_tolerance > 0.f) ? req->gjk_tolerance : 1e-6f;
  p.epa_tol = (req && req->epa_tolerance > 0.f) ? req->epa_tolerance : 1e-6f;
  p.gjk_max_iter = (req && req->gjk_max_iterations) ? (int)req->gjk_max_iterations : 128;
  p.epa_max_iter = (req && req->epa_max_iterations) ? (int)req->epa_max_iterations : 255;
  p.epa_max_faces = (req && req->epa_max_faces) ? (int)req->epa_max_faces : 256;
  const uint32_t fl = req ? req->flags : 0u;
  const bool boolean_only = (fl & FCLG_REQ_BOOLEAN_ONLY) != 0;
  p.want_distance = (distance_query || !boolean_only) ? 1 : 0;
  p.want_epa = (!boolean_only && !(fl & FCLG_REQ_NO_EPA)) ? 1 : 0;
  // fcl::collide without contact runs MPR (gjk_solver-inl.h:86-97); a learned
  // warm start applies to GJK only, so it keeps the GJK boolean
  p.use_mpr = (!distance_query && boolean_only && !(fl & FCLG_REQ_WARM_START) && !(fl & FCLG_REQ_GJK_BOOLEAN)) ? 1 : 0;
  // fcl::collide answers sphere pairs in closed form (gjk_solver-inl.h:209-218);
  // shapeSignedDistance (the distance entry points) has no such path
  p.analytic = (!distance_query && !(fl & FCLG_REQ_NO_ANALYTIC)) ? 1 : 0;
  p.directed = 0;
  p.incremental = 0;
  // a learned start keeps a pair only with a separation certificate found
  // within warm_probe supports and a distance certified to warm_gap
  p.warm_probe = (req && req->warm_probe) ? (int)req->warm_probe : kWarmProbeDefault;
  p.warm_gap = (req && req->warm_gap > 0.f) ? req->warm_gap : kWarmGapDefault;
  return p;
}

int collect_times(fclg_context* c) {
  if (!c->ev_pending) return FCLG_OK;
  FCLG_CUDA(c, cudaEventSynchronize(c->ev[c->ev_epa ? 2 : 1]));
  float a = 0, b = 0;
  FCLG_CUDA(c, cudaEventElapsedTime(&a, c->ev[0], c->ev[1]));
  if (c->ev_epa) FCLG_CUDA(c, cudaEventElapsedTime(&b, c->ev[1], c->ev[2]));
  c->gjk_ms += a;
  c->epa_ms += b;
  c->timed += 1;
  c->ev_pending = false;
  return FCLG_OK;
}

int run_query(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request* req, fclg_result* d_results,
              cudaStream_t st, bool distance_query) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_results) return fail(c, FCLG_E_INVALID, "null pair or result pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  const fclg::QueryParams prm = make_params(req, distance_query);
  if (prm.want_epa) {
    const int rc = ensure_epa(c, n);
    if (rc) return rc;
  }
  fclg::BatchArgs b = batch_args(c);
  b.pairs = reinterpret_cast<const float4*>(d_pairs);
  b.guess = nullptr;
  b.results = reinterpret_cast<float4*>(d_results);
  b.n_pairs = n;
  b.n_shapes = c->n_shapes;
  fclg::EpaQueue q{c->epa_count, c->epa_list, c->epa_rec};
  q.next = c->epa_count + 2;
  if (c->profiling) {
    const int rc = collect_times(c);
    if (rc) return rc;
  }
  FCLG_CUDA(c, cudaMemsetAsync(c->epa_count, 0, kQueueCounters * sizeof(uint32_t), st));
  if (c->bucketing) {
    const int rc = ensure_bucket(c, n);
    if (rc) return rc;
  }
  if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[0], st));
  if (req && (req->flags & FCLG_REQ_WARM_START)) {
    // the model's directions are part of the GJK pass's time
    if (!c->ws) return fail(c, FCLG_E_INVALID, "FCLG_REQ_WARM_START without a model (fclg_set_warmstart)");
    const int rc = ensure_guess(c, n);
    if (rc) return rc;
    FCLG_CUDA(c, fclg::warmstart_predict(c->ws, b.pairs, n, c->guess, st));
    b.guess = c->guess;
    c->launches += 1;
  }
  if (c->bucketing) {
    fclg::BucketScratch bs{c->bk_keys, c->bk_order, c->bk_small, c->bk_small + fclg::kBucketKeys,
                           c->bk_small + 2 * fclg::kBucketKeys};
    FCLG_CUDA(c, fclg::launch_bucketing(b, bs, (uint32_t)c->large_hull, st));
    const int blocks = c->num_sms * c->gjk_ctas_per_sm;
    const fclg::DistList dl{c->epa_count + 6, c->bk_dist, c->epa_count + 7,
                            c->epa_count + 8, c->bk_redo, c->epa_count + 9};
    FCLG_CUDA(c, fclg::launch_gjk(b, prm, q, c->gjk_lanes, bs.order, bs.ranges, blocks, st, c->gjk_refill,
                                  c->epa_count + 4, &dl));
    FCLG_CUDA(c, fclg::launch_gjk(b, prm, q, c->gjk_lanes_large, bs.order, bs.ranges + 2, blocks, st,
                                  c->gjk_refill, c->epa_count + 5));
    c->launches += 4 + fclg::gjk_split_launches(b, prm, c->gjk_lanes, blocks, c->gjk_refill);
  } else {
    FCLG_CUDA(c, fclg::launch_gjk(b, prm, q, c->gjk_lanes, nullptr, nullptr, 0, st, c->gjk_refill));
    c->launches += 1;
  }
  if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[1], st));
  if (prm.want_epa) {
    fclg::EpaQueue ovf{c->epa_count + 1, c->epa_ovf, reinterpret_cast<float4*>(c->epa_resume),
                       c->epa_resume_on ? c->epa_resume_cap : 0u, c->epa_count + 3};
    FCLG_CUDA(c, fclg::launch_epa(b, prm, q, ovf, c->num_sms, c->epa_ctas_per_sm, st));
    c->launches += (uint64_t)fclg::epa_launches(prm);
    if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[2], st));
  }
  if (c->profiling) {
    c->ev_pending = true;
    c->ev_epa = prm.want_epa != 0;
  }
  return FCLG_OK;
}

int run_host_query(fclg_context* c, const fclg_pair* pairs, uint32_t n, const fclg_request* req,
                   fclg_result* results, bool distance_query) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!pairs || !results) return fail(c, FCLG_E_INVALID, "null pair or result pointer");
  int rc = ensure_io(c, n);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(c->io_pairs, pairs, (size_t)n * sizeof(fclg_pair), cudaMemcpyHostToDevice, c->stream));
  rc = run_query(c, static_cast<const fclg_pair*>(c->io_pairs), n, req, static_cast<fclg_result*>(c->io_results),
                 c->stream, distance_query);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(results, c->io_results, (size_t)n * sizeof(fclg_result), cudaMemcpyDeviceToHost,
                               c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}

}  // namespace

extern "C" {

int fclg_version(void) { return 100; }

int fclg_built_arch(void) { return 1030; }

int fclg_create(fclg_context** out, int device) {
  if (!out) return FCLG_E_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return FCLG_E_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FCLG_E_NO_DEVICE;
  if (prop.major * 10 + prop.minor != 103) return FCLG_E_NO_DEVICE;
  fclg_context* c = new fclg_context();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->epa_count, kQueueCounters * sizeof(uint32_t)) != cudaSuccess ||
      fclg::prepare_epa() != cudaSuccess) {
    fclg_destroy(c);
    return FCLG_E_CUDA;
  }
  *out = c;
  return FCLG_OK;
}

void fclg_destroy(fclg_context* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  release_shapes(c);
  if (c->epa_count) cudaFree(c->epa_count);
  if (c->epa_list) cudaFree(c->epa_list);
  if (c->epa_ovf) cudaFree(c->epa_ovf);
  if (c->epa_resume) cudaFree(c->epa_resume);
  if (c->epa_rec) cudaFree(c->epa_rec);
  if (c->io_pairs) cudaFree(c->io_pairs);
  if (c->io_results) cudaFree(c->io_results);
  if (c->bk_keys) cudaFree(c->bk_keys);
  if (c->bk_order) cudaFree(c->bk_order);
  if (c->bk_small) cudaFree(c->bk_small);
  if (c->bk_dist) cudaFree(c->bk_dist);
  if (c->bk_redo) cudaFree(c->bk_redo);
  if (c->mesh_io) cudaFree(c->mesh_io);
  if (c->mesh_cbuf) cudaFree(c->mesh_cbuf);
  if (c->mesh_ctr) cudaFree(c->mesh_ctr);
  if (c->mesh_take) cudaFree(c->mesh_take);
  if (c->contact_take) cudaFree(c->contact_take);
  if (c->guess) cudaFree(c->guess);
  if (c->bp_scratch) cudaFree(c->bp_scratch);
  if (c->bp_io) cudaFree(c->bp_io);
  if (c->bp_join) cudaFree(c->bp_join);
  if (c->hull_aabb) cudaFree(c->hull_aabb);
  if (c->ccd_disp) cudaFree(c->ccd_disp);
  if (c->stream) cudaStreamDestroy(c->stream);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  delete c;
}

const char* fclg_last_error(const fclg_context* c) { return c ? c->err.c_str() : "null context"; }

int fclg_set_shapes(fclg_context* c, const fclg_shape* shapes, uint32_t n_shapes, const float* vertices,
                    uint64_t n_vertices) {
  if (!c) return FCLG_E_INVALID;
  if (!shapes || n_shapes == 0) return fail(c, FCLG_E_INVALID, "no shapes");
  if (n_vertices > 0 && !vertices) return fail(c, FCLG_E_INVALID, "null vertex pointer");
  int rc = validate_shapes(c, shapes, n_shapes, n_vertices);
  if (rc) return rc;
  FCLG_CUDA(c, cudaSetDevice(c->device));
  release_shapes(c);
  FCLG_CUDA(c, cudaMalloc(&c->own_shapes, (size_t)n_shapes * sizeof(fclg_shape)));
  FCLG_CUDA(c, cudaMalloc(&c->own_verts, std::max<uint64_t>(n_vertices, 1) * 4 * sizeof(float)));
  FCLG_CUDA(c, cudaMemcpy(c->own_shapes, shapes, (size_t)n_shapes * sizeof(fclg_shape), cudaMemcpyHostToDevice));
  if (n_vertices)
    FCLG_CUDA(c, cudaMemcpy(c->own_verts, vertices, n_vertices * 4 * sizeof(float), cudaMemcpyHostToDevice));
  c->shapes = static_cast<const int4*>(c->own_shapes);
  c->verts = static_cast<const float4*>(c->own_verts);
  c->n_shapes = n_shapes;
  c->n_verts = n_vertices;
  return build_walks(c, shapes, n_shapes, vertices);
}

int fclg_hull_graph(const float* xyzw, uint32_t nv, uint32_t* starts, uint32_t* first, uint32_t* adj,
                    uint32_t adj_cap, uint32_t* adj_len) {
  if (!xyzw || !starts || !first || !adj_len) return FCLG_E_INVALID;
  fclg::HullGraph g;
  if (!fclg::hull_graph(xyzw, nv, g)) return FCLG_E_INVALID;
  *adj_len = (uint32_t)g.adj.size();
  std::copy(g.start, g.start + 6, starts);
  std::copy(g.first.begin(), g.first.end(), first);
  if (!adj) return FCLG_OK;
  if (adj_cap < g.adj.size()) return FCLG_E_TOO_LARGE;
  std::copy(g.adj.begin(), g.adj.end(), adj);
  return FCLG_OK;
}

int fclg_set_shapes_device(fclg_context* c, const fclg_shape* d_shapes, uint32_t n_shapes, const float* d_vertices,
                           uint64_t n_vertices) {
  if (!c) return FCLG_E_INVALID;
  if (!d_shapes || n_shapes == 0 || !d_vertices) return fail(c, FCLG_E_INVALID, "null shape or vertex pointer");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  // validate the table once on the host: kernels trust vertex ranges
  std::vector<fclg_shape> h(n_shapes);
  FCLG_CUDA(c, cudaMemcpy(h.data(), d_shapes, (size_t)n_shapes * sizeof(fclg_shape), cudaMemcpyDeviceToHost));
  const int rc = validate_shapes(c, h.data(), n_shapes, n_vertices);
  if (rc) return rc;
  release_shapes(c);
  c->shapes = reinterpret_cast<const int4*>(d_shapes);
  c->verts = reinterpret_cast<const float4*>(d_vertices);
  c->n_shapes = n_shapes;
  c->n_verts = n_vertices;
  bool walks = false;
  for (uint32_t i = 0; i < n_shapes && !walks; ++i)
    walks = h[i].type == FCLG_CONVEX && h[i].vert_count > fclg::kWalkMinVertices;
  if (!walks) return FCLG_OK;
  std::vector<float> hv(4 * (size_t)n_vertices);
  FCLG_CUDA(c, cudaMemcpy(hv.data(), d_vertices, hv.size() * sizeof(float), cudaMemcpyDeviceToHost));
  return build_walks(c, h.data(), n_shapes, hv.data());
}

int fclg_distance(fclg_context* c, const fclg_pair* pairs, uint32_t n, const fclg_request* req,
                  fclg_result* results) {
  return run_host_query(c, pairs, n, req, results, true);
}

int fclg_distance_device(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request* req,
                         fclg_result* d_results, void* stream) {
  return run_query(c, d_pairs, n, req, d_results, static_cast<cudaStream_t>(stream), true);
}

int fclg_collide(fclg_context* c, const fclg_pair* pairs, uint32_t n, const fclg_request* req, fclg_result* results) {
  return run_host_query(c, pairs, n, req, results, false);
}

int fclg_collide_device(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request* req,
                        fclg_result* d_results, void* stream) {
  return run_query(c, d_pairs, n, req, d_results, static_cast<cudaStream_t>(stream), false);
}

int fclg_distance64_device(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request64* req,
                           fclg_result64* d_results, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_results) return fail(c, FCLG_E_INVALID, "null pair or result pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  fclg::BatchArgs b = batch_args(c);
  b.pairs = reinterpret_cast<const float4*>(d_pairs);
  b.guess = nullptr;
  b.results = nullptr;
  b.n_pairs = n;
  b.n_shapes = c->n_shapes;
  const double tol = (req && req->gjk_tolerance > 0.) ? req->gjk_tolerance : 1e-6;
  const int max_iter = (req && req->gjk_max_iterations) ? (int)req->gjk_max_iterations : 128;
  FCLG_CUDA(c, fclg::launch_gjk64(b, tol, max_iter, reinterpret_cast<double*>(d_results), c->num_sms * 16,
                                  static_cast<cudaStream_t>(stream)));
  c->launches += 1;
  return FCLG_OK;
}

int fclg_distance64(fclg_context* c, const fclg_pair* pairs, uint32_t n, const fclg_request64* req,
                    fclg_result64* results) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!pairs || !results) return fail(c, FCLG_E_INVALID, "null pair or result pointer");
  // the staging of FP32 results, sized up to hold the 64-byte records
  int rc = ensure_io(c, ((size_t)n * sizeof(fclg_result64) + sizeof(fclg_result) - 1) / sizeof(fclg_result));
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(c->io_pairs, pairs, (size_t)n * sizeof(fclg_pair), cudaMemcpyHostToDevice, c->stream));
  rc = fclg_distance64_device(c, static_cast<const fclg_pair*>(c->io_pairs), n, req,
                              static_cast<fclg_result64*>(c->io_results), c->stream);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(results, c->io_results, (size_t)n * sizeof(fclg_result64), cudaMemcpyDeviceToHost,
                               c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}

int fclg_set_warmstart(fclg_context* c, fclg_warmstart* model) {
  if (!c) return FCLG_E_INVALID;
  if (model && fclg::warmstart_device(model) != c->device)
    return fail(c, FCLG_E_INVALID, "warm-start model lives on another device");
  c->ws = model;
  return FCLG_OK;
}

static bool valid_lanes(int l) { return l == 1 || l == 2 || l == 4 || l == 8 || l == 16 || l == 32; }

int fclg_set_tuning(fclg_context* c, const fclg_tuning* t) {
  if (!c || !t) return FCLG_E_INVALID;
  if ((t->gjk_lanes_small && !valid_lanes(t->gjk_lanes_small)) ||
      (t->gjk_lanes_large && !valid_lanes(t->gjk_lanes_large)))
    return fail(c, FCLG_E_INVALID, "GJK lanes per pair must be 1, 2, 4, 8, 16 or 32");
  if (t->gjk_ctas_per_sm < 0 || t->gjk_ctas_per_sm > 32 || t->epa_ctas_per_sm < 0 || t->epa_ctas_per_sm > 32)
    return fail(c, FCLG_E_INVALID, "CTAs per SM out of range");
  if (t->large_hull_vertices < 0) return fail(c, FCLG_E_INVALID, "negative hull size threshold");
  if (t->bucketing) c->bucketing = t->bucketing > 0;
  if (t->gjk_lanes_small) c->gjk_lanes = t->gjk_lanes_small;
  if (t->gjk_lanes_large) c->gjk_lanes_large = t->gjk_lanes_large;
  if (t->large_hull_vertices) c->large_hull = t->large_hull_vertices;
  if (t->gjk_ctas_per_sm) c->gjk_ctas_per_sm = t->gjk_ctas_per_sm;
  if (t->epa_ctas_per_sm) c->epa_ctas_per_sm = t->epa_ctas_per_sm;
  if (t->support_walk) c->support_walk = t->support_walk > 0;
  if (t->gjk_refill) c->gjk_refill = t->gjk_refill > 0;
  if (t->epa_resume) c->epa_resume_on = t->epa_resume > 0;
  return FCLG_OK;
}

int fclg_get_tuning(const fclg_context* c, fclg_tuning* t) {
  if (!c || !t) return FCLG_E_INVALID;
  t->bucketing = c->bucketing ? 1 : -1;
  t->gjk_lanes_small = c->gjk_lanes;
  t->gjk_lanes_large = c->gjk_lanes_large;
  t->large_hull_vertices = c->large_hull;
  t->gjk_ctas_per_sm = c->gjk_ctas_per_sm;
  t->epa_ctas_per_sm = c->epa_ctas_per_sm;
  t->support_walk = c->support_walk ? 1 : -1;
  t->gjk_refill = c->gjk_refill ? 1 : -1;
  t->epa_resume = c->epa_resume_on ? 1 : -1;
  return FCLG_OK;
}

int fclg_set_launch(fclg_context* c, int gjk_lanes, int epa_ctas_per_sm) {
  fclg_tuning t{};
  t.gjk_lanes_small = gjk_lanes;
  t.gjk_lanes_large = gjk_lanes;
  t.epa_ctas_per_sm = epa_ctas_per_sm;
  return fclg_set_tuning(c, &t);
}

uint64_t fclg_launch_count(const fclg_context* c) { return c ? c->launches : 0; }

int fclg_bvh_build(const float* vertices, uint32_t nv, const int32_t* tris, uint32_t nt, fclg_mesh_node* nodes,
                   float* tris_xyzw) {
  if (!vertices || !tris || !nodes || !tris_xyzw || nv == 0 || nt == 0 || nt > (1u << 29)) return FCLG_E_INVALID;
  std::vector<fclg::MeshNodeRec> nn;
  std::vector<float> soup;
  if (fclg::build_obb_bvh(vertices, nv, tris, nt, nn, soup) != 0) return FCLG_E_INVALID;
  std::memcpy(nodes, nn.data(), nn.size() * sizeof(fclg::MeshNodeRec));
  std::memcpy(tris_xyzw, soup.data(), soup.size() * sizeof(float));
  return FCLG_OK;
}

int fclg_bvh_node_sizes(const float* vertices, uint32_t nv, const int32_t* tris, uint32_t nt, double* sizes,
                        uint32_t* depth) {
  if (!vertices || !tris || nv == 0 || nt == 0 || nt > (1u << 29)) return FCLG_E_INVALID;
  std::vector<fclg::MeshNodeRec> nn;
  std::vector<float> soup;
  std::vector<double> sz;
  uint32_t d = 0;
  if (fclg::build_obb_bvh(vertices, nv, tris, nt, nn, soup, &sz, &d) != 0) return FCLG_E_INVALID;
  if (sizes) std::memcpy(sizes, sz.data(), sz.size() * sizeof(double));
  if (depth) *depth = d;
  return FCLG_OK;
}

int fclg_mesh_create(fclg_context* c, const float* vertices, uint32_t nv, const int32_t* tris, uint32_t nt,
                     fclg_mesh** out) {
  if (!c) return FCLG_E_INVALID;
  if (!out || !vertices || !tris || nv == 0 || nt == 0) return fail(c, FCLG_E_INVALID, "empty mesh or null pointer");
  *out = nullptr;
  if (nt > (1u << 29)) return fail(c, FCLG_E_TOO_LARGE, "too many triangles");
  std::vector<fclg::MeshNodeRec> nodes;
  std::vector<float> soup;
  std::vector<double> sizes;
  uint32_t depth = 0;
  const int rc = fclg::build_obb_bvh(vertices, nv, tris, nt, nodes, soup, &sizes, &depth);
  if (rc == -2) return fail(c, FCLG_E_INVALID, "triangle vertex index out of range");
  if (rc) return fail(c, FCLG_E_INVALID, "empty mesh");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  fclg_mesh* m = new fclg_mesh();
  m->device = c->device;
  m->n_nodes = (uint32_t)nodes.size();
  m->n_tris = nt;
  m->depth = depth;
  cudaError_t e = cudaMalloc(&m->nodes, nodes.size() * sizeof(fclg::MeshNodeRec));
  if (e == cudaSuccess) e = cudaMalloc(&m->tris, soup.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->sizes, sizes.size() * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMemcpy(m->nodes, nodes.data(), nodes.size() * sizeof(fclg::MeshNodeRec), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->tris, soup.data(), soup.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->sizes, sizes.data(), sizes.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    fclg_mesh_destroy(m);
    return cuda_fail(c, e, "mesh upload");
  }
  *out = m;
  return FCLG_OK;
}

void fclg_mesh_destroy(fclg_mesh* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->nodes) cudaFree(m->nodes);
  if (m->tris) cudaFree(m->tris);
  if (m->sizes) cudaFree(m->sizes);
  delete m;
}

int fclg_mesh_info(const fclg_mesh* m, uint32_t* n_nodes, uint32_t* n_tris) {
  if (!m) return FCLG_E_INVALID;
  if (n_nodes) *n_nodes = m->n_nodes;
  if (n_tris) *n_tris = m->n_tris;
  return FCLG_OK;
}

int fclg_mesh_export(const fclg_mesh* m, fclg_mesh_node* nodes, float* tris) {
  if (!m) return FCLG_E_INVALID;
  if (cudaSetDevice(m->device) != cudaSuccess) return FCLG_E_CUDA;
  if (nodes && cudaMemcpy(nodes, m->nodes, (size_t)m->n_nodes * 64, cudaMemcpyDeviceToHost) != cudaSuccess)
    return FCLG_E_CUDA;
  if (tris && cudaMemcpy(tris, m->tris, (size_t)m->n_tris * 48, cudaMemcpyDeviceToHost) != cudaSuccess)
    return FCLG_E_CUDA;
  return FCLG_OK;
}

int fclg_mesh_collide_device(fclg_context* c, const fclg_mesh* a, const fclg_mesh* b, const float* d_poses,
                             uint32_t n, uint32_t max_contacts, uint8_t* d_flags, uint32_t* d_counts, int32_t* d_pairs,
                             uint32_t* d_status, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (!a || !b) return fail(c, FCLG_E_INVALID, "null mesh");
  if (n == 0) return FCLG_OK;
  if (max_contacts == 0) return fail(c, FCLG_E_INVALID, "max_contacts must be >= 1");
  if (!d_poses || !d_flags || !d_counts || !d_pairs) return fail(c, FCLG_E_INVALID, "null pointer");
  if (a->device != c->device || b->device != c->device) return fail(c, FCLG_E_INVALID, "mesh on another device");
  // the traversal orders node pairs by a 64-bit path key: one bit per descent
  if (a->depth + b->depth > 62) return fail(c, FCLG_E_TOO_LARGE, "BVH depths sum above 62");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  fclg::MeshArgs m;
  m.a = fclg::MeshDev{static_cast<const float4*>(a->nodes), static_cast<const float4*>(a->tris), a->n_nodes, a->n_tris,
                      static_cast<const double*>(a->sizes)};
  m.b = fclg::MeshDev{static_cast<const float4*>(b->nodes), static_cast<const float4*>(b->tris), b->n_nodes, b->n_tris,
                      static_cast<const double*>(b->sizes)};
  m.poses = reinterpret_cast<const float4*>(d_poses);
  m.n_poses = n;
  m.max_contacts = max_contacts;
  m.flags = d_flags;
  m.counts = d_counts;
  m.pairs = d_pairs;
  m.status = d_status;
  // a persistent grid whose warps take poses from a counter
  const int blocks = fclg::mesh_collide_resident_blocks(c->num_sms);
  if (!c->mesh_take) FCLG_CUDA(c, cudaMalloc(&c->mesh_take, sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMemsetAsync(c->mesh_take, 0, sizeof(uint32_t), static_cast<cudaStream_t>(stream)));
  m.next = c->mesh_take;
  const int cbuf_len = fclg::mesh_contact_buffer_len(max_contacts);
  if (cbuf_len > 0) {
    // contact buffers in device memory, one per warp of the grid
    const size_t need = (size_t)fclg::mesh_collide_warps(blocks) * cbuf_len * (8 + 8);
    if (need > ((size_t)8 << 30))
      return fail(c, FCLG_E_TOO_LARGE, "max_contacts too large for the ordered contact buffers (8 GiB)");
    if (need > c->mesh_cbuf_bytes) {
      if (c->mesh_cbuf) cudaFree(c->mesh_cbuf);
      c->mesh_cbuf = nullptr;
      c->mesh_cbuf_bytes = 0;
      FCLG_CUDA(c, cudaMalloc(&c->mesh_cbuf, need));
      c->mesh_cbuf_bytes = need;
    }
    const size_t n_entries = (size_t)fclg::mesh_collide_warps(blocks) * cbuf_len;
    m.cbuf_key = static_cast<unsigned long long*>(c->mesh_cbuf);
    m.cbuf_pair = reinterpret_cast<int2*>(static_cast<char*>(c->mesh_cbuf) + n_entries * 8);
    m.cbuf_len = (uint32_t)cbuf_len;
  }
  if (c->profiling) {
    if (!c->mesh_ctr) {
      FCLG_CUDA(c, cudaMalloc(&c->mesh_ctr, 2 * sizeof(unsigned long long)));
      FCLG_CUDA(c, cudaMemset(c->mesh_ctr, 0, 2 * sizeof(unsigned long long)));
    }
    m.counters = c->mesh_ctr;
  }
  clear_pending_error();
  FCLG_CUDA(c, fclg::launch_mesh_collide(m, blocks, static_cast<cudaStream_t>(stream)));
  c->launches += 1;
  return FCLG_OK;
}

int fclg_mesh_traffic(fclg_context* c, uint64_t* node_pairs, uint64_t* triangle_pairs, int reset) {
  if (!c) return FCLG_E_INVALID;
  unsigned long long h[2] = {0, 0};
  if (c->mesh_ctr) {
    FCLG_CUDA(c, cudaSetDevice(c->device));
    FCLG_CUDA(c, cudaDeviceSynchronize());
    FCLG_CUDA(c, cudaMemcpy(h, c->mesh_ctr, sizeof h, cudaMemcpyDeviceToHost));
    if (reset) FCLG_CUDA(c, cudaMemset(c->mesh_ctr, 0, sizeof h));
  }
  if (node_pairs) *node_pairs = h[0];
  if (triangle_pairs) *triangle_pairs = h[1];
  return FCLG_OK;
}

int fclg_mesh_collide(fclg_context* c, const fclg_mesh* a, const fclg_mesh* b, const float* poses, uint32_t n,
                      uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* pairs, uint32_t* status) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!poses || !flags || !counts || !pairs) return fail(c, FCLG_E_INVALID, "null pointer");
  if (max_contacts == 0) return fail(c, FCLG_E_INVALID, "max_contacts must be >= 1");
  auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  const size_t b_poses = up16((size_t)n * 48), b_flags = up16(n), b_counts = up16((size_t)n * 4),
               b_pairs = up16((size_t)n * max_contacts * 8), b_status = up16((size_t)n * 4);
  const size_t need = b_poses + b_flags + b_counts + b_pairs + b_status;
  if (need > c->mesh_io_bytes) {
    if (c->mesh_io) cudaFree(c->mesh_io);
    c->mesh_io = nullptr;
    c->mesh_io_bytes = 0;
    FCLG_CUDA(c, cudaSetDevice(c->device));
    FCLG_CUDA(c, cudaMalloc(&c->mesh_io, need));
    c->mesh_io_bytes = need;
  }
  char* base = static_cast<char*>(c->mesh_io);
  float* d_poses = reinterpret_cast<float*>(base);
  uint8_t* d_flags = reinterpret_cast<uint8_t*>(base + b_poses);
  uint32_t* d_counts = reinterpret_cast<uint32_t*>(base + b_poses + b_flags);
  int32_t* d_pairs = reinterpret_cast<int32_t*>(base + b_poses + b_flags + b_counts);
  uint32_t* d_status = reinterpret_cast<uint32_t*>(base + b_poses + b_flags + b_counts + b_pairs);
  FCLG_CUDA(c, cudaMemcpyAsync(d_poses, poses, (size_t)n * 48, cudaMemcpyHostToDevice, c->stream));
  const int rc = fclg_mesh_collide_device(c, a, b, d_poses, n, max_contacts, d_flags, d_counts, d_pairs, d_status,
                                          c->stream);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(flags, d_flags, n, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(counts, d_counts, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(pairs, d_pairs, (size_t)n * max_contacts * 8, cudaMemcpyDeviceToHost, c->stream));
  if (status) FCLG_CUDA(c, cudaMemcpyAsync(status, d_status, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}

static int run_mesh_shape(fclg_context* c, const fclg_mesh* mesh, const uint32_t* d_shape_ids, const float* d_poses,
                          uint32_t n, uint32_t max_contacts, uint8_t* d_flags, uint32_t* d_counts, int32_t* d_tri_ids,
                          float* d_contacts, uint32_t* d_status, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (!mesh) return fail(c, FCLG_E_INVALID, "null mesh");
  if (n == 0) return FCLG_OK;
  if (max_contacts == 0) return fail(c, FCLG_E_INVALID, "max_contacts must be >= 1");
  if (!d_shape_ids || !d_poses || !d_flags || !d_counts || !d_tri_ids) return fail(c, FCLG_E_INVALID, "null pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  if (mesh->device != c->device) return fail(c, FCLG_E_INVALID, "mesh on another device");
  // the traversal orders nodes by a 64-bit path key: one bit per descent
  if (mesh->depth > 62) return fail(c, FCLG_E_TOO_LARGE, "BVH depth above 62");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  fclg::MeshShapeArgs m;
  m.mesh = fclg::MeshDev{static_cast<const float4*>(mesh->nodes), static_cast<const float4*>(mesh->tris),
                         mesh->n_nodes, mesh->n_tris, static_cast<const double*>(mesh->sizes)};
  m.shapes = c->shapes;
  m.verts = c->verts;
  m.n_shapes = c->n_shapes;
  m.shape_ids = d_shape_ids;
  m.poses = reinterpret_cast<const float4*>(d_poses);
  m.n = n;
  m.max_contacts = max_contacts;
  m.gjk_tol = 1e-6f;
  m.gjk_max_iter = 128;
  m.flags = d_flags;
  m.counts = d_counts;
  m.tri_ids = d_tri_ids;
  m.status = d_status;
  m.contacts = d_contacts;
  // a persistent grid whose warps take queries from a counter
  const int blocks = fclg::mesh_shape_resident_blocks(c->num_sms, d_contacts != nullptr);
  if (!c->mesh_take) FCLG_CUDA(c, cudaMalloc(&c->mesh_take, sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMemsetAsync(c->mesh_take, 0, sizeof(uint32_t), static_cast<cudaStream_t>(stream)));
  m.next = c->mesh_take;
  const int cbuf_len = fclg::mesh_contact_buffer_len(max_contacts);
  if (cbuf_len > 0) {
    // contact buffers in device memory, one per warp of the grid
    const size_t n_entries = (size_t)fclg::mesh_shape_warps(blocks) * cbuf_len;
    if (n_entries * 16 > ((size_t)8 << 30))
      return fail(c, FCLG_E_TOO_LARGE, "max_contacts too large for the ordered contact buffers (8 GiB)");
    if (n_entries * 16 > c->mesh_cbuf_bytes) {
      if (c->mesh_cbuf) cudaFree(c->mesh_cbuf);
      c->mesh_cbuf = nullptr;
      c->mesh_cbuf_bytes = 0;
      FCLG_CUDA(c, cudaMalloc(&c->mesh_cbuf, n_entries * 16));
      c->mesh_cbuf_bytes = n_entries * 16;
    }
    m.cbuf_key = static_cast<unsigned long long*>(c->mesh_cbuf);
    m.cbuf_val = reinterpret_cast<int2*>(static_cast<char*>(c->mesh_cbuf) + n_entries * 8);
    m.cbuf_len = (uint32_t)cbuf_len;
  }
  clear_pending_error();
  FCLG_CUDA(c, fclg::launch_mesh_shape(m, blocks, static_cast<cudaStream_t>(stream)));
  c->launches += 1;
  if (d_contacts) {
    if (!c->contact_take) FCLG_CUDA(c, cudaMalloc(&c->contact_take, sizeof(uint32_t)));
    FCLG_CUDA(c, cudaMemsetAsync(c->contact_take, 0, sizeof(uint32_t), static_cast<cudaStream_t>(stream)));
    m.contact_next = c->contact_take;
    FCLG_CUDA(c, fclg::launch_mesh_contacts(m, c->num_sms, static_cast<cudaStream_t>(stream)));
    c->launches += 1;
  }
  return FCLG_OK;
}

int fclg_mesh_shape_collide_device(fclg_context* c, const fclg_mesh* mesh, const uint32_t* d_shape_ids,
                                   const float* d_poses, uint32_t n, uint32_t max_contacts, uint8_t* d_flags,
                                   uint32_t* d_counts, int32_t* d_tri_ids, uint32_t* d_status, void* stream) {
  return run_mesh_shape(c, mesh, d_shape_ids, d_poses, n, max_contacts, d_flags, d_counts, d_tri_ids, nullptr,
                        d_status, stream);
}

int fclg_mesh_shape_contacts_device(fclg_context* c, const fclg_mesh* mesh, const uint32_t* d_shape_ids,
                                    const float* d_poses, uint32_t n, uint32_t max_contacts, uint8_t* d_flags,
                                    uint32_t* d_counts, int32_t* d_tri_ids, float* d_contacts, uint32_t* d_status,
                                    void* stream) {
  if (c && n && !d_contacts) return fail(c, FCLG_E_INVALID, "null contact pointer");
  return run_mesh_shape(c, mesh, d_shape_ids, d_poses, n, max_contacts, d_flags, d_counts, d_tri_ids, d_contacts,
                        d_status, stream);
}

static int mesh_shape_host(fclg_context* c, const fclg_mesh* mesh, const uint32_t* shape_ids, const float* poses,
                           uint32_t n, uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* tri_ids,
                           float* contacts, uint32_t* status) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!shape_ids || !poses || !flags || !counts || !tri_ids) return fail(c, FCLG_E_INVALID, "null pointer");
  if (max_contacts == 0) return fail(c, FCLG_E_INVALID, "max_contacts must be >= 1");
  auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  const size_t b_poses = up16((size_t)n * 48), b_ids = up16((size_t)n * 4), b_flags = up16(n),
               b_counts = up16((size_t)n * 4), b_tris = up16((size_t)n * max_contacts * 4),
               b_status = up16((size_t)n * 4), b_contacts = contacts ? up16((size_t)n * max_contacts * 32) : 0;
  const size_t need = b_poses + b_ids + b_flags + b_counts + b_tris + b_status + b_contacts;
  if (need > c->mesh_io_bytes) {
    if (c->mesh_io) cudaFree(c->mesh_io);
    c->mesh_io = nullptr;
    c->mesh_io_bytes = 0;
    FCLG_CUDA(c, cudaSetDevice(c->device));
    FCLG_CUDA(c, cudaMalloc(&c->mesh_io, need));
    c->mesh_io_bytes = need;
  }
  char* p = static_cast<char*>(c->mesh_io);
  float* d_poses = reinterpret_cast<float*>(p);
  uint32_t* d_ids = reinterpret_cast<uint32_t*>(p += b_poses);
  uint8_t* d_flags = reinterpret_cast<uint8_t*>(p += b_ids);
  uint32_t* d_counts = reinterpret_cast<uint32_t*>(p += b_flags);
  int32_t* d_tris = reinterpret_cast<int32_t*>(p += b_counts);
  uint32_t* d_status = reinterpret_cast<uint32_t*>(p += b_tris);
  float* d_contacts = contacts ? reinterpret_cast<float*>(p += b_status) : nullptr;
  FCLG_CUDA(c, cudaMemcpyAsync(d_poses, poses, (size_t)n * 48, cudaMemcpyHostToDevice, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(d_ids, shape_ids, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  const int rc = run_mesh_shape(c, mesh, d_ids, d_poses, n, max_contacts, d_flags, d_counts, d_tris, d_contacts,
                                d_status, c->stream);
  if (rc) return rc;
  if (contacts)
    FCLG_CUDA(c, cudaMemcpyAsync(contacts, d_contacts, (size_t)n * max_contacts * 32, cudaMemcpyDeviceToHost,
                                 c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(flags, d_flags, n, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(counts, d_counts, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(tri_ids, d_tris, (size_t)n * max_contacts * 4, cudaMemcpyDeviceToHost, c->stream));
  if (status) FCLG_CUDA(c, cudaMemcpyAsync(status, d_status, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}

int fclg_mesh_shape_collide(fclg_context* c, const fclg_mesh* mesh, const uint32_t* shape_ids, const float* poses,
                            uint32_t n, uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* tri_ids,
                            uint32_t* status) {
  return mesh_shape_host(c, mesh, shape_ids, poses, n, max_contacts, flags, counts, tri_ids, nullptr, status);
}

int fclg_mesh_shape_contacts(fclg_context* c, const fclg_mesh* mesh, const uint32_t* shape_ids, const float* poses,
                             uint32_t n, uint32_t max_contacts, uint8_t* flags, uint32_t* counts, int32_t* tri_ids,
                             float* contacts, uint32_t* status) {
  if (c && n && !contacts) return fail(c, FCLG_E_INVALID, "null contact pointer");
  return mesh_shape_host(c, mesh, shape_ids, poses, n, max_contacts, flags, counts, tri_ids, contacts, status);
}

// ---------------------------------------------------------------------------
// Broadphase (BinaryAABB_Tree::SelfCollision over CollisionObject AABBs).
// ---------------------------------------------------------------------------

int fclg_broadphase_device(fclg_context* c, const uint32_t* d_shape_ids, const float* d_poses, uint32_t n,
                           uint32_t* d_pairs, uint32_t cap, uint32_t* d_n_pairs, float* d_aabb_lo, float* d_aabb_hi,
                           void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (!d_n_pairs || (n && (!d_shape_ids || !d_poses)) || (cap && !d_pairs))
    return fail(c, FCLG_E_INVALID, "null pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  const size_t need = fclg::broadphase_scratch_bytes(n, c->n_shapes);
  if (need > c->bp_bytes) {
    if (c->bp_scratch) cudaFree(c->bp_scratch);
    c->bp_scratch = nullptr;
    c->bp_bytes = 0;
    FCLG_CUDA(c, cudaMalloc(&c->bp_scratch, need));
    c->bp_bytes = need;
  }
  fclg::BroadphaseArgs a;
  a.shapes = c->shapes;
  a.verts = c->verts;
  a.n_shapes = c->n_shapes;
  a.shape_ids = d_shape_ids;
  a.poses = reinterpret_cast<const float4*>(d_poses);
  a.n = n;
  a.pairs = d_pairs;
  a.cap = cap;
  a.count = d_n_pairs;
  a.aabb_lo = reinterpret_cast<float4*>(d_aabb_lo);
  a.aabb_hi = reinterpret_cast<float4*>(d_aabb_hi);
  a.split = 0;
  clear_pending_error();
  FCLG_CUDA(c, fclg::launch_broadphase(a, c->bp_scratch, static_cast<cudaStream_t>(stream)));
  c->launches += n ? (uint64_t)fclg::broadphase_launches() : 0;
  return FCLG_OK;
}

int fclg_broadphase_cross_device(fclg_context* c, const uint32_t* d_ids_a, const float* d_poses_a, uint32_t n_a,
                                 const uint32_t* d_ids_b, const float* d_poses_b, uint32_t n_b, uint32_t* d_pairs,
                                 uint32_t cap, uint32_t* d_n_pairs, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (!d_n_pairs || (n_a && (!d_ids_a || !d_poses_a)) || (n_b && (!d_ids_b || !d_poses_b)) || (cap && !d_pairs))
    return fail(c, FCLG_E_INVALID, "null pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t n = n_a + n_b;
  if (n_a == 0 || n_b == 0) {
    FCLG_CUDA(c, cudaMemsetAsync(d_n_pairs, 0, 4, st));
    return FCLG_OK;
  }
  const size_t b_ids = ((size_t)n * 4 + 255) & ~(size_t)255;
  const size_t need = b_ids + (size_t)n * 48;
  if (need > c->bp_join_bytes) {
    if (c->bp_join) cudaFree(c->bp_join);
    c->bp_join = nullptr;
    c->bp_join_bytes = 0;
    FCLG_CUDA(c, cudaMalloc(&c->bp_join, need));
    c->bp_join_bytes = need;
  }
  uint32_t* ids = static_cast<uint32_t*>(c->bp_join);
  float* poses = reinterpret_cast<float*>(static_cast<char*>(c->bp_join) + b_ids);
  FCLG_CUDA(c, cudaMemcpyAsync(ids, d_ids_a, (size_t)n_a * 4, cudaMemcpyDeviceToDevice, st));
  FCLG_CUDA(c, cudaMemcpyAsync(ids + n_a, d_ids_b, (size_t)n_b * 4, cudaMemcpyDeviceToDevice, st));
  FCLG_CUDA(c, cudaMemcpyAsync(poses, d_poses_a, (size_t)n_a * 48, cudaMemcpyDeviceToDevice, st));
  FCLG_CUDA(c, cudaMemcpyAsync(poses + 12 * (size_t)n_a, d_poses_b, (size_t)n_b * 48, cudaMemcpyDeviceToDevice, st));
  const size_t scratch = fclg::broadphase_scratch_bytes(n, c->n_shapes);
  if (scratch > c->bp_bytes) {
    if (c->bp_scratch) cudaFree(c->bp_scratch);
    c->bp_scratch = nullptr;
    c->bp_bytes = 0;
    FCLG_CUDA(c, cudaMalloc(&c->bp_scratch, scratch));
    c->bp_bytes = scratch;
  }
  fclg::BroadphaseArgs a;
  a.shapes = c->shapes;
  a.verts = c->verts;
  a.n_shapes = c->n_shapes;
  a.shape_ids = ids;
  a.poses = reinterpret_cast<const float4*>(poses);
  a.n = n;
  a.pairs = d_pairs;
  a.cap = cap;
  a.count = d_n_pairs;
  a.aabb_lo = nullptr;
  a.aabb_hi = nullptr;
  a.split = n_a;
  clear_pending_error();
  FCLG_CUDA(c, fclg::launch_broadphase(a, c->bp_scratch, st));
  c->launches += (uint64_t)fclg::broadphase_launches();
  return FCLG_OK;
}

int fclg_broadphase(fclg_context* c, const uint32_t* shape_ids, const float* poses, uint32_t n, uint32_t* pairs,
                    uint32_t cap, uint32_t* n_pairs, float* aabbs) {
  if (!c) return FCLG_E_INVALID;
  if (!n_pairs || (n && (!shape_ids || !poses)) || (cap && !pairs)) return fail(c, FCLG_E_INVALID, "null pointer");
  auto up256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_ids = up256((size_t)n * 4), b_poses = up256((size_t)n * 48), b_pairs = up256((size_t)cap * 8),
               b_box = up256((size_t)n * 16), b_cnt = 256;
  const size_t need = b_ids + b_poses + b_pairs + 2 * b_box + b_cnt;
  FCLG_CUDA(c, cudaSetDevice(c->device));
  if (need > c->bp_io_bytes) {
    if (c->bp_io) cudaFree(c->bp_io);
    c->bp_io = nullptr;
    c->bp_io_bytes = 0;
    FCLG_CUDA(c, cudaMalloc(&c->bp_io, need));
    c->bp_io_bytes = need;
  }
  char* p = static_cast<char*>(c->bp_io);
  uint32_t* d_ids = reinterpret_cast<uint32_t*>(p);
  float* d_poses = reinterpret_cast<float*>(p += b_ids);
  uint32_t* d_pairs = reinterpret_cast<uint32_t*>(p += b_poses);
  float* d_lo = reinterpret_cast<float*>(p += b_pairs);
  float* d_hi = reinterpret_cast<float*>(p += b_box);
  uint32_t* d_cnt = reinterpret_cast<uint32_t*>(p += b_box);
  if (n) {
    FCLG_CUDA(c, cudaMemcpyAsync(d_ids, shape_ids, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    FCLG_CUDA(c, cudaMemcpyAsync(d_poses, poses, (size_t)n * 48, cudaMemcpyHostToDevice, c->stream));
  }
  const int rc = fclg_broadphase_device(c, d_ids, d_poses, n, d_pairs, cap, d_cnt, d_lo, d_hi, c->stream);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(n_pairs, d_cnt, 4, cudaMemcpyDeviceToHost, c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  const uint32_t got = std::min(*n_pairs, cap);
  if (got) FCLG_CUDA(c, cudaMemcpy(pairs, d_pairs, (size_t)got * 8, cudaMemcpyDeviceToHost));
  if (aabbs && n) {
    std::vector<float> lo(4 * (size_t)n), hi(4 * (size_t)n);
    FCLG_CUDA(c, cudaMemcpy(lo.data(), d_lo, lo.size() * 4, cudaMemcpyDeviceToHost));
    FCLG_CUDA(c, cudaMemcpy(hi.data(), d_hi, hi.size() * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) {
        aabbs[6 * i + k] = lo[4 * i + k];
        aabbs[6 * i + 3 + k] = hi[4 * i + k];
      }
  }
  return FCLG_OK;
}

int fclg_object_pairs_device(fclg_context* c, const uint32_t* d_shape_ids, const float* d_poses,
                             const uint32_t* d_candidates, uint32_t m, fclg_pair* d_pairs, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (m && (!d_shape_ids || !d_poses || !d_candidates || !d_pairs)) return fail(c, FCLG_E_INVALID, "null pointer");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  FCLG_CUDA(c, fclg::launch_object_pairs(d_shape_ids, d_poses, d_candidates, m, d_pairs,
                                         static_cast<cudaStream_t>(stream)));
  c->launches += m ? 1 : 0;
  return FCLG_OK;
}

int fclg_set_profiling(fclg_context* c, int enable) {
  if (!c) return FCLG_E_INVALID;
  FCLG_CUDA(c, cudaSetDevice(c->device));
  if (enable && !c->ev[0])
    for (auto& e : c->ev) FCLG_CUDA(c, cudaEventCreate(&e));
  c->profiling = enable != 0;
  return FCLG_OK;
}

int fclg_pass_times(fclg_context* c, double* gjk_ms, double* epa_ms, uint64_t* queries, int reset) {
  if (!c) return FCLG_E_INVALID;
  const int rc = collect_times(c);
  if (rc) return rc;
  if (gjk_ms) *gjk_ms = c->gjk_ms;
  if (epa_ms) *epa_ms = c->epa_ms;
  if (queries) *queries = c->timed;
  if (reset) {
    c->gjk_ms = c->epa_ms = 0;
    c->timed = 0;
  }
  return FCLG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Scratch-free signed distance: fclg_distance_device_static.
//
// The same GJK + EPA passes as fclg_distance_device (unbucketed launch: every
// pair with the context's small-pair GJK lane count), but the EPA queue lives
// in the file-scope device array below instead of context buffers grown with
// cudaMalloc, so a call allocates nothing.  Layout of the array:
//   [0, 256)                         counts[2]: EPA work list, overflow list
//   [256, +4 * kStaticMax)           work list (pair indices)
//   [.., +4 * kStaticMax)            overflow list (work-list items)
//   [.., +kEpaRecordBytes * kStaticMax)  final GJK simplex per work-list item (then its final-solve record)
// counts must be zero before the GJK pass; each call zeroes them with
// cudaMemsetAsync on its stream (the lists and records are written before
// they are read and need no clearing).
//
// Set-up: the first call on a device (with that device current) looks the
// array up with cudaGetSymbolAddress and caches the address for the device;
// later calls only read the cache.  Make the first call before any stream
// capture.  Every call on a device shares the one array, so calls that
// overlap in time on that device (other streams, other contexts, other host
// threads) race on it: order them on one stream, or join them by events.
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kStaticMax = FCLG_STATIC_MAX_PAIRS;
constexpr size_t kStaticHeadBytes = 256;
constexpr size_t kStaticListOffset = kStaticHeadBytes;
constexpr size_t kStaticOvfOffset = kStaticListOffset + kStaticMax * sizeof(uint32_t);
constexpr size_t kStaticRecOffset = kStaticOvfOffset + kStaticMax * sizeof(uint32_t);
constexpr size_t kStaticBytes = kStaticRecOffset + kStaticMax * fclg::kEpaRecordBytes;
static_assert(kStaticRecOffset % 16 == 0, "simplex records hold float4");
constexpr int kStaticMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

namespace {

std::mutex g_static_mutex;
unsigned char* g_static_base[kStaticMaxDevices] = {};

// Address of g_static_scratch on the current device (c->device), looked up on
// the first call for that device and cached per device ordinal.  The address
// belongs to the device's primary context (the one the runtime API uses): a
// cudaDeviceReset, or another context made current on the device, makes the
// cached address stale, so this entry point must not be used across either.
int static_scratch(fclg_context* c, unsigned char** out) {
  if (c->device < 0 || c->device >= kStaticMaxDevices) return fail(c, FCLG_E_INVALID, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_base[c->device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetSymbolAddress(g_static_scratch)");
    g_static_base[c->device] = static_cast<unsigned char*>(p);
  }
  *out = g_static_base[c->device];
  return FCLG_OK;
}

}  // namespace

extern "C" int fclg_distance_device_static(fclg_context* c, const fclg_pair* d_pairs, uint32_t n,
                                           const fclg_request* req, fclg_result* d_results, void* stream) {
  if (!c) return FCLG_E_INVALID;
  if (n > kStaticMax) {
    char b[160];
    snprintf(b, sizeof b, "fclg_distance_device_static: %u pairs exceed its fixed scratch of %u pairs per call", n,
             (unsigned)kStaticMax);
    return fail(c, FCLG_E_TOO_LARGE, b);
  }
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_results) return fail(c, FCLG_E_INVALID, "null pair or result pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  if (req && (req->flags & FCLG_REQ_WARM_START))
    return fail(c, FCLG_E_INVALID, "fclg_distance_device_static: FCLG_REQ_WARM_START needs per-pair scratch");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  unsigned char* base = nullptr;
  const int rc = static_scratch(c, &base);
  if (rc) return rc;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const fclg::QueryParams prm = make_params(req, true);
  fclg::BatchArgs b = batch_args(c);
  b.pairs = reinterpret_cast<const float4*>(d_pairs);
  b.guess = nullptr;
  b.results = reinterpret_cast<float4*>(d_results);
  b.n_pairs = n;
  b.n_shapes = c->n_shapes;
  uint32_t* counts = reinterpret_cast<uint32_t*>(base);
  fclg::EpaQueue q{counts, reinterpret_cast<uint32_t*>(base + kStaticListOffset),
                   reinterpret_cast<float4*>(base + kStaticRecOffset)};
  q.next = counts + 2;
  if (c->profiling) {  // the pass times of fclg_pass_times cover these calls too
    const int prc = collect_times(c);
    if (prc) return prc;
  }
  if (prm.want_epa) FCLG_CUDA(c, cudaMemsetAsync(counts, 0, kQueueCounters * sizeof(uint32_t), st));
  if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[0], st));
  FCLG_CUDA(c, fclg::launch_gjk(b, prm, q, c->gjk_lanes, nullptr, nullptr, 0, st, c->gjk_refill));
  c->launches += 1;
  if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[1], st));
  if (prm.want_epa) {
    fclg::EpaQueue ovf{counts + 1, reinterpret_cast<uint32_t*>(base + kStaticOvfOffset), nullptr, 0u, counts + 3};
    FCLG_CUDA(c, fclg::launch_epa(b, prm, q, ovf, c->num_sms, c->epa_ctas_per_sm, st));
    c->launches += (uint64_t)fclg::epa_launches(prm);
    if (c->profiling) FCLG_CUDA(c, cudaEventRecord(c->ev[2], st));
  }
  if (c->profiling) {
    c->ev_pending = true;
    c->ev_epa = prm.want_epa != 0;
  }
  return FCLG_OK;
}

// ---------------------------------------------------------------------------
// fcl::collide in the directed penetration mode (useDirectedPenetration).
// ---------------------------------------------------------------------------

namespace {

int run_directed(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const float* d_dirs, const fclg_request* req,
                 fclg_result* d_results, cudaStream_t st) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  const bool learned = req && (req->flags & FCLG_REQ_WARM_START);
  if (!d_pairs || (!d_dirs && !learned) || !d_results)
    return fail(c, FCLG_E_INVALID, "null pair, direction or result pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  if (learned && !(req->flags & FCLG_REQ_INCREMENTAL))
    return fail(c, FCLG_E_INVALID, "a learned direction seeds the incremental mode only (FCLG_REQ_INCREMENTAL)");
  if (learned && !c->ws) return fail(c, FCLG_E_INVALID, "FCLG_REQ_WARM_START without a model (fclg_set_warmstart)");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  if (learned) {
    // the model's directions are the hints: the incremental mode seeded by the learned direction
    const int rc = ensure_guess(c, n);
    if (rc) return rc;
    FCLG_CUDA(c, fclg::warmstart_predict(c->ws, reinterpret_cast<const float4*>(d_pairs), n, c->guess, st));
    c->launches += 1;
    d_dirs = c->guess;
  }
  fclg::QueryParams prm = make_params(req, false);
  prm.want_epa = 0;
  prm.use_mpr = 0;
  prm.analytic = 0;
  prm.directed = 1;
  prm.incremental = (req && (req->flags & FCLG_REQ_INCREMENTAL)) ? 1 : 0;
  fclg::BatchArgs b = batch_args(c);
  b.pairs = reinterpret_cast<const float4*>(d_pairs);
  b.guess = d_dirs;
  b.results = reinterpret_cast<float4*>(d_results);
  b.n_pairs = n;
  b.n_shapes = c->n_shapes;
  FCLG_CUDA(c, fclg::launch_directed(b, prm, c->num_sms * c->gjk_ctas_per_sm, st));
  c->launches += 1;
  return FCLG_OK;
}

}  // namespace

extern "C" int fclg_collide_directed_device(fclg_context* c, const fclg_pair* d_pairs, uint32_t n,
                                            const float* d_dirs, const fclg_request* req, fclg_result* d_results,
                                            void* stream) {
  return run_directed(c, d_pairs, n, d_dirs, req, d_results, static_cast<cudaStream_t>(stream));
}

extern "C" int fclg_collide_directed(fclg_context* c, const fclg_pair* pairs, uint32_t n, const float* dirs,
                                     const fclg_request* req, fclg_result* results) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  const bool learned = req && (req->flags & FCLG_REQ_WARM_START);
  if (!pairs || (!dirs && !learned) || !results) return fail(c, FCLG_E_INVALID, "null pair, direction or result pointer");
  int rc = ensure_io(c, n);
  if (!rc) rc = ensure_guess(c, n);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(c->io_pairs, pairs, (size_t)n * sizeof(fclg_pair), cudaMemcpyHostToDevice, c->stream));
  if (!learned)
    FCLG_CUDA(c, cudaMemcpyAsync(c->guess, dirs, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  rc = run_directed(c, static_cast<const fclg_pair*>(c->io_pairs), n, learned ? nullptr : c->guess, req,
                    static_cast<fclg_result*>(c->io_results), c->stream);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(results, c->io_results, (size_t)n * sizeof(fclg_result), cudaMemcpyDeviceToHost,
                               c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs of a whole query, and the launch-shape autotuner.
// ---------------------------------------------------------------------------

struct fclg_graph {
  int device = 0;
  const fclg_context* ctx = nullptr;
  uint64_t epoch = 0;
  uint64_t launches = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

// Allocates every scratch buffer a query of n pairs needs, so that a capture
// or a timed loop allocates nothing.
int reserve_query(fclg_context* c, uint32_t n, const fclg_request* req, bool distance_query) {
  const fclg::QueryParams prm = make_params(req, distance_query);
  int rc = FCLG_OK;
  if (prm.want_epa) rc = ensure_epa(c, n);
  if (!rc && c->bucketing) rc = ensure_bucket(c, n);
  if (!rc && req && (req->flags & FCLG_REQ_WARM_START)) rc = ensure_guess(c, n);
  return rc;
}

}  // namespace

extern "C" int fclg_graph_create(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request* req,
                                 fclg_result* d_results, int distance_query, fclg_graph** out) {
  if (!c || !out) return FCLG_E_INVALID;
  *out = nullptr;
  if (n == 0 || !d_pairs || !d_results) return fail(c, FCLG_E_INVALID, "graph of an empty or null batch");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  int rc = reserve_query(c, n, req, distance_query != 0);
  if (rc) return rc;
  cudaStream_t cs = nullptr;
  FCLG_CUDA(c, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  const bool prof = c->profiling;
  c->profiling = false;
  const uint64_t l0 = c->launches;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  cudaGraph_t g = nullptr;
  if (e == cudaSuccess) {
    rc = run_query(c, d_pairs, n, req, d_results, cs, distance_query != 0);
    e = cudaStreamEndCapture(cs, &g);
  }
  c->profiling = prof;
  const uint64_t launches = c->launches - l0;
  c->launches = l0;
  cudaStreamDestroy(cs);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return rc ? rc : cuda_fail(c, e, "stream capture of a query");
  }
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(c, e, "cudaGraphInstantiate");
  }
  fclg_graph* G = new fclg_graph();
  G->device = c->device;
  G->ctx = c;
  G->epoch = c->scratch_epoch;
  G->launches = launches;
  G->graph = g;
  G->exec = ex;
  *out = G;
  return FCLG_OK;
}

extern "C" int fclg_graph_launch(fclg_context* c, fclg_graph* g, void* stream) {
  if (!c || !g || g->ctx != c) return fail(c, FCLG_E_INVALID, "graph of another context");
  if (g->epoch != c->scratch_epoch)
    return fail(c, FCLG_E_INVALID, "graph is stale: the context reallocated its query scratch since the capture");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  FCLG_CUDA(c, cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
  c->launches += g->launches;
  return FCLG_OK;
}

extern "C" void fclg_graph_destroy(fclg_graph* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

extern "C" int fclg_autotune(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_request* req,
                             fclg_result* d_results, int distance_query, fclg_tuning* best, float* best_ms) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0 || !d_pairs || !d_results) return fail(c, FCLG_E_INVALID, "autotune on an empty or null batch");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  FCLG_CUDA(c, cudaSetDevice(c->device));
  fclg_tuning keep{};
  fclg_get_tuning(c, &keep);
  const bool prof = c->profiling;
  c->profiling = false;
  // candidates: GJK lanes for small / large hulls, the hull split, bucketing
  std::vector<fclg_tuning> cand;
  // (the support walk only changes one-lane launches, and only when hulls have walk blocks)
  for (int ls : {1, 2, 4, 8})
    for (int ll : {1, 4, 8, 16})
      for (int lh : {64, 128, 256})
        for (int walk : {1, -1})
          for (int refill : {1, -1}) {
            // the walk and the refilling kernel only change one-lane launches
            if (ls != 1 && ll != 1 && (walk < 0 || refill < 0)) continue;
            if (walk < 0 && !c->walk_tab) continue;
            fclg_tuning t = keep;
            t.bucketing = 1;
            t.gjk_lanes_small = ls;
            t.gjk_lanes_large = ll;
            t.large_hull_vertices = lh;
            t.support_walk = walk;
            t.gjk_refill = refill;
            cand.push_back(t);
          }
  {
    fclg_tuning t = keep;
    t.bucketing = -1;
    t.gjk_lanes_small = 1;
    cand.push_back(t);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FCLG_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    rc = fail(c, FCLG_E_CUDA, "cudaEventCreate");
  float best_t = 0.f;
  fclg_tuning best_c = keep;
  for (size_t i = 0; i < cand.size() && rc == FCLG_OK; ++i) {
    rc = fclg_set_tuning(c, &cand[i]);
    if (!rc) rc = reserve_query(c, n, req, distance_query != 0);
    if (!rc) rc = run_query(c, d_pairs, n, req, d_results, c->stream, distance_query != 0);  // warm-up
    if (rc) break;
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < 2 && !rc; ++r) rc = run_query(c, d_pairs, n, req, d_results, c->stream, distance_query != 0);
    cudaEventRecord(e1, c->stream);
    if (rc) break;
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = fail(c, FCLG_E_CUDA, "autotune timing");
      break;
    }
    ms *= 0.5f;
    if (i == 0 || ms < best_t) {
      best_t = ms;
      best_c = cand[i];
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  c->profiling = prof;
  fclg_set_tuning(c, rc ? &keep : &best_c);
  if (rc) return rc;
  if (best) fclg_get_tuning(c, best);
  if (best_ms) *best_ms = best_t;
  return FCLG_OK;
}

// ---------------------------------------------------------------------------
// Translational continuous collision of shape pairs.
// ---------------------------------------------------------------------------

static_assert(sizeof(fclg_displacement) == 16, "displacement layout (read as float4)");
static_assert(sizeof(fclg_ccd_result) == 16, "ccd result layout (written as float4)");
static_assert(sizeof(fclg_ccd_request) == 24, "ccd request layout");
static_assert(sizeof(fclg_ccd_result) <= sizeof(fclg_result), "ccd results share the query result staging");
static_assert(sizeof(fclg_result64) == 64, "fclg_result64 layout (written as 8 doubles)");
static_assert(sizeof(fclg_request64) == 16, "fclg_request64 layout");

namespace {

int run_ccd(fclg_context* c, const fclg_pair* d_pairs, uint32_t n, const fclg_displacement* d_disp,
            const fclg_ccd_request* req, fclg_ccd_result* d_results, cudaStream_t st) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!d_pairs || !d_disp || !d_results) return fail(c, FCLG_E_INVALID, "null pair, displacement or result pointer");
  if (!c->shapes) return fail(c, FCLG_E_NO_SHAPES, "no shapes set");
  fclg::CcdParams prm;
  prm.toc_type = req ? (int)req->toc_type : fclg::kTocNone;
  if (prm.toc_type < fclg::kTocNone || prm.toc_type > fclg::kTocSample)
    return fail(c, FCLG_E_INVALID, "toc_type is not one of FCLG_TOC_*");
  prm.max_iter = (req && req->max_gjk_iterations > 0) ? req->max_gjk_iterations : 128;
  prm.tol = (req && req->gjk_tolerance > 0.f) ? req->gjk_tolerance : 1e-6f;
  prm.zero_tol = (req && req->zero_movement_tolerance > 0.0) ? req->zero_movement_tolerance : 1e-4;
  FCLG_CUDA(c, cudaSetDevice(c->device));
  clear_pending_error();
  if (prm.toc_type == fclg::kTocBox && !c->hull_aabb_valid) {
    if (!c->hull_aabb) FCLG_CUDA(c, cudaMalloc(&c->hull_aabb, (size_t)c->n_shapes * 2 * sizeof(float4)));
    FCLG_CUDA(c, fclg::launch_hull_aabbs(c->shapes, c->verts, c->n_shapes, c->hull_aabb, st));
    c->launches += 1;
    c->hull_aabb_valid = true;
  }
  fclg::BatchArgs b = batch_args(c);
  b.pairs = reinterpret_cast<const float4*>(d_pairs);
  b.results = nullptr;
  b.n_pairs = n;
  b.n_shapes = c->n_shapes;
  const uint32_t* order = nullptr;
  if (c->bucketing) {
    // shape-class order, as the distance query sorts its pairs
    const int rc = ensure_bucket(c, n);
    if (rc) return rc;
    fclg::BucketScratch bs{c->bk_keys, c->bk_order, c->bk_small, c->bk_small + fclg::kBucketKeys,
                           c->bk_small + 2 * fclg::kBucketKeys};
    FCLG_CUDA(c, fclg::launch_bucketing(b, bs, (uint32_t)c->large_hull, st));
    c->launches += 3;
    order = bs.order;
  }
  if (!c->mesh_take) FCLG_CUDA(c, cudaMalloc(&c->mesh_take, sizeof(uint32_t)));
  FCLG_CUDA(c, cudaMemsetAsync(c->mesh_take, 0, sizeof(uint32_t), st));
  FCLG_CUDA(c, fclg::launch_ccd(b, reinterpret_cast<const float4*>(d_disp), c->hull_aabb, prm, order,
                                reinterpret_cast<float4*>(d_results), c->num_sms, st, c->mesh_take));
  c->launches += 1;
  return FCLG_OK;
}

}  // namespace

extern "C" int fclg_translational_ccd_device(fclg_context* c, const fclg_pair* d_pairs, uint32_t n,
                                             const fclg_displacement* d_disp, const fclg_ccd_request* req,
                                             fclg_ccd_result* d_results, void* stream) {
  return run_ccd(c, d_pairs, n, d_disp, req, d_results, static_cast<cudaStream_t>(stream));
}

extern "C" int fclg_translational_ccd(fclg_context* c, const fclg_pair* pairs, uint32_t n,
                                      const fclg_displacement* disp, const fclg_ccd_request* req,
                                      fclg_ccd_result* results) {
  if (!c) return FCLG_E_INVALID;
  if (n == 0) return FCLG_OK;
  if (!pairs || !disp || !results) return fail(c, FCLG_E_INVALID, "null pair, displacement or result pointer");
  int rc = ensure_io(c, n);
  if (rc) return rc;
  if (n > c->ccd_disp_cap) {
    if (c->ccd_disp) cudaFree(c->ccd_disp);
    c->ccd_disp = nullptr;
    c->ccd_disp_cap = 0;
    const size_t cap = std::max<size_t>(n, 1024);
    FCLG_CUDA(c, cudaMalloc(&c->ccd_disp, cap * sizeof(fclg_displacement)));
    c->ccd_disp_cap = cap;
  }
  FCLG_CUDA(c, cudaMemcpyAsync(c->io_pairs, pairs, (size_t)n * sizeof(fclg_pair), cudaMemcpyHostToDevice, c->stream));
  FCLG_CUDA(c, cudaMemcpyAsync(c->ccd_disp, disp, (size_t)n * sizeof(fclg_displacement), cudaMemcpyHostToDevice,
                               c->stream));
  // the results (16 bytes each) fit the staging of query results
  rc = run_ccd(c, static_cast<const fclg_pair*>(c->io_pairs), n, static_cast<const fclg_displacement*>(c->ccd_disp),
               req, static_cast<fclg_ccd_result*>(c->io_results), c->stream);
  if (rc) return rc;
  FCLG_CUDA(c, cudaMemcpyAsync(results, c->io_results, (size_t)n * sizeof(fclg_ccd_result), cudaMemcpyDeviceToHost,
                               c->stream));
  FCLG_CUDA(c, cudaStreamSynchronize(c->stream));
  return FCLG_OK;
}
