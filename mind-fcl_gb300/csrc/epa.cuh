// EPA penetration depth / witness points, one warp per overlapping pair, with
// the polytope held in the warp's slice of shared memory.
//
// Algorithm (epa.hpp:133-237 and the polytope code it drives): repeatedly take
// the face nearest the origin, evaluate the support along its outward normal,
// stop when the support point is within the tolerance of that face's plane,
// else remove the patch of faces the new point sees — grown from the nearest
// face through visible neighbours, as computeVisiblePatch's DFS does
// (epa_polytope_expand.hpp:120-180) — and fan new faces from the point to the
// patch's horizon.  Capacity (live faces <= max_faces, the reference's
// MallocFailed) and the iteration limit end the loop with the current nearest
// face, as the reference does.  A face counts as seen when the point lies
// beyond its plane by more than a tenth of the tolerance (the reference uses
// >= 0): faces coplanar at FP32 resolution stay, which keeps the polytope
// convex where supports tie exactly.
//
// Faces are ranked by plane distance among those the origin projects into
// (the reference's pointToTriangle witness_in_simplex, epa_polytope_utils.h:
// 88-165); among coplanar triangles that picks the one holding the nearest
// point.
//
// GPU layout: per iteration the work is proportional to the visible patch,
// not to the polytope: the patch grows in frontier rounds (a lane per frontier
// face, classification claimed with a compare-and-swap on a per-iteration
// stamp), horizon edges are recorded by the same rounds (a patch face's edge
// whose neighbour ends hidden), slots are recycled through a free stack, and
// the fan is linked through a per-vertex "edge starting here" table.  Only the nearest-face argmin touches every
// slot: one shared-memory load per lane per 32 slots.  Face planes are FP32
// unit normals and distances whose cross products are compensated (see
// face_plane); the final closest-face solve (depth, barycentric witness
// points) runs in FP64 (epa_final_solve), in the batched query a thread per
// pair after the EPA launches (epa_pass.cu) rather than on one lane of the
// warp that ran the pair.
//
// Initial polytope from the GJK simplex: epa_simplex2polytope.hpp:41-376
// (touching detection, triangle blown up along +-normal, segment search over
// 72 directions, tetrahedron).
#pragma once
#include "support.cuh"

#ifndef FCLG_EPA_TRACE
#define FCLG_EPA_TRACE(...) \
  do {                      \
  } while (0)
#endif
// Phase-timing hook (cycle counts per EPA phase when defined by a profiling
// build; nothing by default).
#ifndef FCLG_EPA_PHASE
#define FCLG_EPA_PHASE(k) \
  do {                    \
  } while (0)
#endif

namespace fclg {

constexpr uint32_t kNoSlot = 0xFFFFFFFFu;
// EPA outcome internal to the two-layout scheme: the polytope outgrew the
// small layout; the pair is rerun in the large one.
constexpr int kEpaOverflow = 16;
// A face counts as seen by a new point lying more than kVisEps * tolerance
// beyond its plane: above FP32 rounding of the plane test, far below the
// convergence tolerance.
constexpr float kVisEps = 0.1f;

// A pair's support data, one copy per warp in shared memory (read by
// broadcast) instead of one per lane in local memory.
struct EpaPairData {
  ShapeDev A, B;
  Pose pose;
  const float4* verts;
};

// Support of A - B (MinkowskiSupport<32>'s) over the warp, reading the pair
// from shared memory.
struct SharedSupport32 {
  const EpaPairData* d;
  __device__ __forceinline__ void operator()(f3 dir, f3& pa, f3& pb) const {
    const Group<32> g = Group<32>::make();
    const ShapeDev A = d->A, B = d->B;
    const Pose X = d->pose;
    pa = shape_support<32>(A, d->verts, dir, g);
    pb = X.apply(shape_support<32>(B, d->verts, X.rotT(-dir), g));
  }
};

template <int FMAX, int VMAX>
struct EpaSmem {
  float4 fn[FMAX];         // outward unit normal xyz, plane distance (inf: dead or degenerate)
  float fkey[FMAX];        // selection key: plane distance, + tolerance when the origin projects outside
  uint32_t fv[FMAX];       // vertex indices v0 | v1 << 8 | v2 << 16, counter-clockwise seen from outside
  uint16_t fadj[FMAX][4];  // neighbour across edge k = (v_k, v_k+1)
  uint32_t fmark[FMAX];    // classification stamp of the current expansion
  float4 vw[VMAX];         // Minkowski vertex w = pa - pb
  float4 vpa[VMAX];        // support point on shape a
  uint32_t start_at[VMAX];
  uint16_t patch[FMAX];    // faces of the visible patch, in discovery order
  uint16_t freestk[FMAX];  // recycled face slots
  uint16_t hz_s[FMAX + 8];  // horizon edge: patch face (a simple horizon has at most
  uint8_t hz_e[FMAX + 8];   // patch size + 2 edges) and its edge index
  uint16_t hz_slot[FMAX + 8];
  uint32_t npatch;
  uint32_t nhz;             // horizon edges found by the flood fill
  EpaPairData pair;         // the pair being run (SharedSupport32)
};

__device__ __forceinline__ uint32_t fvert(uint32_t packed, int k) { return (packed >> (8 * k)) & 0xFFu; }
__device__ __forceinline__ f3 ld3(const float4& q) { return mk3(q.x, q.y, q.z); }

// a * b - c * d to within about one rounding of the exact value (Kahan's
// difference of products with one FMA recovering the rounding of c * d).
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) {
  const float w = c * d;
  const float e = fmaf(-c, d, w);
  const float f = fmaf(a, b, -w);
  return f + e;
}

// Face plane (outward unit normal, distance from the origin).  The edge
// vectors of a face are differences of nearby FP32 vertices, exact or nearly
// so; a plain FP32 cross product of them still loses the digits that give a
// thin face its direction (error ~ eps |e1||e2| / |e1 x e2| radians), enough to
// misjudge which faces a distant support point sees and fold the polytope.
// Each component is therefore formed as a compensated difference of products,
// which keeps the normal accurate to a few FP32 roundings.
__device__ __forceinline__ float4 face_plane(f3 a, f3 b, f3 c) {
  const f3 u = b - a, v = c - a;
  const f3 n = mk3(diff_of_products(u.y, v.z, u.z, v.y), diff_of_products(u.z, v.x, u.x, v.z),
                   diff_of_products(u.x, v.y, u.y, v.x));
  const float n2 = sqn(n);
  if (!(n2 > 0.f)) return make_float4(0.f, 0.f, 0.f, INFINITY);
  const f3 nu = n * rsqrtf(n2);
  return make_float4(nu.x, nu.y, nu.z, dot(nu, a));
}

// Whether the origin's projection onto a face's plane lies inside its
// triangle (barycentric coordinates >= -1e-4).
__device__ __forceinline__ bool projects_inside(f3 a, f3 b, f3 c, float4 plane) {
  if (!(plane.w < INFINITY)) return false;
  const f3 u = ld3(plane);
  const f3 p = u * plane.w;
  const float e0 = dot(u, cross(b - a, p - a));
  const float e1 = dot(u, cross(c - b, p - b));
  const float e2 = dot(u, cross(a - c, p - c));
  const float tot = e0 + e1 + e2;
  const float slack = -1e-4f * fabsf(tot);
  return tot > 0.f && e0 >= slack && e1 >= slack && e2 >= slack;
}

struct EpaResult {
  int status;
  float depth;
  f3 p0, p1;
  int iterations;
  int resume_nv;  // kEpaOverflow: vertices of the polytope state to continue from
  // A warp that defers the final solve (EpaWarp<..., true>) leaves here the
  // final face's vertex indices (packed as EpaSmem::fv; kNoSlot when the
  // result needs no solve) and in p0 / p1 the fallback support pair; the
  // caller runs epa_final_solve on that face's vertices.
  uint32_t fin_fv;
};

// Byte offsets of a polytope state written by a layout of F faces / V
// vertices when it runs out of slots (the state before the iteration that
// did not fit), read back by a larger layout, which continues from it: a
// larger layout that had run from the start would hold the same state at the
// same iteration (slots are assigned the same way until the smaller one
// fills), so the answers equal a restart's.
template <int F, int V>
struct EpaResume {
  static constexpr size_t kHead = 0;                  // int nv, hw, live, fs_top, iterations
  static constexpr size_t kFn = 32;                   // float4 [F]
  static constexpr size_t kFkey = kFn + 16 * F;       // float [F]
  static constexpr size_t kFv = kFkey + 4 * F;        // uint32 [F]
  static constexpr size_t kFadj = kFv + 4 * F;        // uint16 [F][4]
  static constexpr size_t kFree = kFadj + 8 * F;      // uint16 [F]
  static constexpr size_t kVw = (kFree + 2 * F + 15) & ~(size_t)15;  // float4 [V]
  static constexpr size_t kVpa = kVw + 16 * V;        // float4 [V]
  static constexpr size_t kBytes = kVpa + 16 * V;
};

// epa_polytope_utils.h:58-86
__device__ __forceinline__ float point_to_line(f3 p, f3 a, f3 b) {
  const f3 ab = b - a;
  const float len = nrm(ab);
  if (len <= 0.f) return nrm(p - a);
  return nrm(cross(p - a, ab)) / len;
}
__device__ __forceinline__ float point_to_plane(f3 p, f3 a, f3 b, f3 c) {
  const f3 n = cross(a - b, b - c);
  const float nl = nrm(n);
  if (nl <= 0.f) return point_to_line(p, a, b);
  return fabsf(dot(n * (1.f / nl), a - p));
}

// DEFER: the final closest-face solve is left to the caller (EpaResult::fin_fv)
// instead of running on lane 0 inside the warp.
template <int FMAX, int VMAX, class Sup = MinkowskiSupport<32>, bool DEFER = false>
struct EpaWarp {
  EpaSmem<FMAX, VMAX>& P;
  const Sup& sup;
  float tol;
  unsigned lane;
  int nv, hw, live, fs_top;
  uint32_t stamp;  // even; advanced by 2 per expansion, never reused by this warp

  __device__ __forceinline__ f3 W(uint32_t i) const { return ld3(P.vw[i]); }

  // Vertices pushed by lane 0; callers __syncwarp before reading them.
  __device__ __forceinline__ void push_vertex(f3 pa, f3 pb) {
    if (lane == 0) {
      const f3 w = pa - pb;
      P.vw[nv] = make_float4(w.x, w.y, w.z, 0.f);
      P.vpa[nv] = make_float4(pa.x, pa.y, pa.z, 0.f);
    }
    ++nv;
  }

  __device__ __forceinline__ void write_face(uint32_t t, uint32_t a, uint32_t b, uint32_t c) {
    const f3 A = W(a), B = W(b), C = W(c);
    const float4 pl = face_plane(A, B, C);
    P.fv[t] = a | (b << 8) | (c << 16);
    P.fn[t] = pl;
    // Selection key: the plane distance, biased by the tolerance when the
    // origin's projection misses the triangle.  The argmin of the key is the
    // nearest face, except that a face the origin projects into wins when it
    // is within the tolerance of the nearest plane: among coplanar triangles
    // it holds the nearest point, and a sliver whose plane is nearest but
    // whose triangle misses the projection is the reference's edge feature.
    P.fkey[t] = projects_inside(A, B, C, pl) ? pl.w : pl.w + tol;
  }

  // Initial polytope from faces (index triples into the vertices already
  // pushed), oriented away from the vertex centroid: a lane per face, then a
  // lane per (face, edge) finding the neighbour across it (nf <= 8).  Returns
  // false when the faces do not close up.
  __device__ bool build_faces(const int (*tri)[3], int nf) {
    if ((int)lane < nf) {
      f3 c = mk3(0, 0, 0);
      for (int i = 0; i < nv; ++i) c = c + W(i);
      c = c * (1.f / (float)nv);
      const int f = (int)lane;
      int i = tri[f][0], j = tri[f][1], k = tri[f][2];
      const f3 n = cross(W(j) - W(i), W(k) - W(i));
      if (dot(n, W(i) - c) < 0.f) { const int t = j; j = k; k = t; }
      write_face(f, i, j, k);
      P.fmark[f] = 0;
    }
    __syncwarp();
    bool ok = true;
    if ((int)lane < 3 * nf) {
      const int f = (int)lane / 3, e = (int)lane % 3;
      const uint32_t u = fvert(P.fv[f], e), v = fvert(P.fv[f], (e + 1) % 3);
      int found = -1;
      for (int g = 0; g < nf && found < 0; ++g) {
        if (g == f) continue;
        for (int h = 0; h < 3; ++h)
          if (fvert(P.fv[g], h) == v && fvert(P.fv[g], (h + 1) % 3) == u) { found = g; break; }
      }
      if (found < 0) ok = false;
      else P.fadj[f][e] = (uint16_t)found;
    }
    __syncwarp();
    hw = nf;
    live = nf;
    fs_top = 0;
    return __all_sync(0xFFFFFFFFu, ok);
  }

  // formNewTetrahedronPolytope, epa_simplex2polytope.hpp:143-174
  __device__ bool tetra() {
    const int tri[4][3] = {{0, 1, 2}, {0, 3, 1}, {1, 3, 2}, {2, 3, 0}};
    return build_faces(tri, 4);
  }

  // The final solve on the face with vertices fvp (epa_final_solve), on lane 0
  // only (the lane that reports the result: the FP64 pipe is narrow), or,
  // deferred, the face and the fallback pair recorded for the caller.
  __device__ void finalize(uint32_t fvp, f3 cand_pa, f3 cand_pb, EpaResult& r) const {
    if constexpr (DEFER) {
      r.fin_fv = fvp;
      r.p0 = cand_pa;
      r.p1 = cand_pb;
      return;
    }
    if (lane != 0) return;
    const uint32_t ia = fvert(fvp, 0), ib = fvert(fvp, 1), ic = fvert(fvp, 2);
    epa_final_solve(W(ia), W(ib), W(ic), ld3(P.vpa[ia]), ld3(P.vpa[ib]), ld3(P.vpa[ic]), cand_pa, cand_pb, r.p0,
                    r.p1, r.depth);
  }

  __device__ void touching(f3 pa, f3 pb, EpaResult& r) const {
    const f3 m = (pa + pb) * 0.5f;
    r.status = kEpaTouching;
    r.depth = 0.f;
    r.p0 = m;
    r.p1 = m;
  }

  // simplexToPolytope3, epa_simplex2polytope.hpp:112-141: vertices 0..2 pushed.
  __device__ bool from_triangle(EpaResult& r, bool& done) {
    const f3 a = W(0), b = W(1), c = W(2);
    f3 n = cross(b - a, c - a);
    if (!(sqn(n) > 0.f)) { r.status = kEpaFailed; done = true; return false; }
    n = normalized(n);
    f3 pa0, pb0, pa1, pb1;
    sup(n, pa0, pb0);
    sup(-n, pa1, pb1);
    const float d0 = point_to_plane(pa0 - pb0, a, b, c);
    const float d1 = point_to_plane(pa1 - pb1, a, b, c);
    if (d0 <= tol) { touching(pa0, pb0, r); done = true; return false; }
    if (d1 <= tol) { touching(pa1, pb1, r); done = true; return false; }
    if (d0 > d1) push_vertex(pa0, pb0);
    else push_vertex(pa1, pb1);
    __syncwarp();
    return tetra();
  }

  // simplexToPolytope2, epa_simplex2polytope.hpp:176-376: vertices 0, 1 pushed.
  __device__ bool from_segment(EpaResult& r, bool& done) {
    const f3 a = W(0), b = W(1);
    const float thr = tol, thr2 = tol * tol;
    const f3 ab = b - a;
    if (sqn(ab) < thr2) { r.status = kEpaFailed; done = true; return false; }
    const f3 abu = normalized(ab);
    f3 dinit = mk3(abu.y, -abu.x, 0.f);
    bool okd = sqn(dinit) > thr2;
    if (!okd) { dinit = mk3(abu.z, 0.f, -abu.x); okd = sqn(dinit) > thr2; }
    if (!okd) { dinit = mk3(0.f, abu.z, -abu.y); okd = sqn(dinit) > thr2; }
    if (!okd) { r.status = kEpaFailed; done = true; return false; }
    dinit = normalized(dinit);
    f3 dcur = dinit, pa, pb;
    bool found = false;
    for (int i = 0; i < 72; ++i) {
      sup(dcur, pa, pb);
      const f3 v = pa - pb;
      if (point_to_line(v, a, b) > thr) { found = true; break; }
      const float step = 2.0f * 3.145926f / 72.0f;  // the reference's constant
      dcur = normalized(dcur + cross(abu, v) * step);
    }
    if (!found) {
      sup(dinit, pa, pb);
      touching(pa, pb, r);
      done = true;
      return false;
    }
    const f3 v0 = pa - pb, v0pa = pa, v0pb = pb;
    f3 pa1, pb1;
    sup(-dcur, pa1, pb1);
    const f3 v1 = pa1 - pb1;
    if (point_to_line(v1, a, b) < thr) { touching(pa1, pb1, r); done = true; return false; }
    const f3 nn = cross(v0 - a, v1 - a);
    if (sqn(nn) < thr2) { r.status = kEpaFailed; done = true; return false; }
    const f3 d2 = normalized(nn);
    f3 pa2, pb2, pa3, pb3;
    sup(d2, pa2, pb2);
    if (point_to_line(pa2 - pb2, a, b) < thr) { touching(pa2, pb2, r); done = true; return false; }
    sup(-d2, pa3, pb3);
    if (point_to_line(pa3 - pb3, a, b) < thr) { touching(pa3, pb3, r); done = true; return false; }
    // The reference's double pyramid: ring a, v0, b, v1 (slots 0, 2, 1, 3)
    // with apexes v2 (slot 4) and v3 (slot 5).
    push_vertex(v0pa, v0pb);
    push_vertex(pa1, pb1);
    push_vertex(pa2, pb2);
    push_vertex(pa3, pb3);
    __syncwarp();
    const int tri[8][3] = {{4, 0, 2}, {4, 2, 1}, {4, 1, 3}, {4, 3, 0}, {5, 0, 2}, {5, 2, 1}, {5, 1, 3}, {5, 3, 0}};
    return build_faces(tri, 8);
  }

  // Warp argmin of the selection key over live faces (ties: lowest slot);
  // returns the slot and its plane distance.
  __device__ __forceinline__ void nearest(int& best_slot, float& best_d) const {
    float bk = INFINITY;
    int bs = 0x7FFFFFFF;
    for (int s = (int)lane; s < hw; s += 32) {
      const float k = P.fkey[s];
      if (k < bk) { bk = k; bs = s; }
    }
    // warp minimum of the key by two reductions: the smallest key (an
    // order-preserving map to unsigned, -0 taken as +0), then the lowest slot
    // holding it
    bk += 0.f;
    const uint32_t kb = __float_as_uint(bk);
    const uint32_t u = (kb & 0x80000000u) ? ~kb : (kb | 0x80000000u);
    const uint32_t umin = __reduce_min_sync(0xFFFFFFFFu, u);
    best_slot = (int)__reduce_min_sync(0xFFFFFFFFu, u == umin ? (uint32_t)bs : 0xFFFFFFFFu);
    best_d = (best_slot != 0x7FFFFFFF) ? P.fn[best_slot].w : INFINITY;
  }

  // One expansion with the new vertex nv-1 from the visible face `start`;
  // returns 0 ok, 1 over max_faces live faces, 2 broken topology, 3 out of
  // face slots in this layout.
  __device__ int expand(int start, int max_faces) {
    const uint32_t vnew = (uint32_t)(nv - 1);
    const f3 w = W(vnew);
    stamp += 2;
    const uint32_t kVis = stamp + 1, kHid = stamp;
    if (lane == 0) {
      P.fmark[start] = kVis;
      P.patch[0] = (uint16_t)start;
      P.npatch = 1;
      P.nhz = 0;
    }
    __syncwarp();
    // Frontier rounds over the visible patch.  Each patch face looks across
    // its three edges; the neighbour's mark is final once read as visible /
    // hidden or once a CAS settled it (ours or another lane's), so an edge
    // whose neighbour ends hidden is a horizon edge and is recorded here.
    FCLG_EPA_PHASE(3);
    int lo = 0, hi = 1;
    for (int round = 0; round < FMAX && lo < hi; ++round) {
      // one (patch face, edge) per lane
      for (int ke = 3 * lo + (int)lane; ke < 3 * hi; ke += 32) {
        const uint32_t f = P.patch[ke / 3];
        {
          const int e = ke % 3;
          const uint32_t g = P.fadj[f][e];
          uint32_t m = P.fmark[g];
          if (m != kVis && m != kHid) {
            const float4 q = P.fn[g];
            const bool visible = dot(ld3(q), w - W(fvert(P.fv[g], 0))) > kVisEps * tol;
            const uint32_t want = visible ? kVis : kHid;
            const uint32_t old = atomicCAS(&P.fmark[g], m, want);
            if (old == m) {
              m = want;
              if (visible) {
                const uint32_t slot = atomicAdd(&P.npatch, 1u);
                if (slot < FMAX) P.patch[slot] = (uint16_t)g;
              }
            } else {
              m = old;  // settled by another lane this expansion
            }
          }
          if (m == kHid) {
            const uint32_t o = atomicAdd(&P.nhz, 1u);
            if (o < FMAX + 8) {
              P.hz_s[o] = (uint16_t)f;
              P.hz_e[o] = (uint8_t)e;
            }
          }
        }
      }
      __syncwarp();
      lo = hi;
      hi = P.npatch < (uint32_t)FMAX ? (int)P.npatch : FMAX;
      __syncwarp();
    }
    const int n_rem = hi;
    const int n_hz = (int)P.nhz;
    FCLG_EPA_PHASE(4);
    if (P.npatch > (uint32_t)FMAX) return 2;
    const int new_live = live - n_rem + n_hz;
    const int avail = fs_top + n_rem;
    const int fresh = n_hz > avail ? n_hz - avail : 0;
    if (n_hz < 3 || n_hz > FMAX + 8) return 2;
    if (new_live > max_faces) return 1;
    if (hw + fresh > FMAX) return 3;
    // recycle the patch's slots (pushed above the older free slots)
    for (int k = (int)lane; k < n_rem; k += 32) P.freestk[fs_top + k] = P.patch[k];
    __syncwarp();
    bool err = false;
    if (n_hz <= 32 && n_rem <= 32) {
      // the usual case, one horizon edge per lane: phases A-C below with the
      // edge in registers
      const int k = (int)lane;
      const bool on = k < n_hz;
      uint32_t a = 0, b = 0, g = 0, t = 0;
      if (on) {
        const uint32_t hs = P.hz_s[k], he = P.hz_e[k];
        const uint32_t fvs = P.fv[hs];
        a = fvert(fvs, (int)he);
        b = fvert(fvs, (int)(he == 2 ? 0 : he + 1));
        g = P.fadj[hs][he];
        t = (k < avail) ? P.freestk[avail - 1 - k] : (uint32_t)(hw + (k - avail));
        P.hz_slot[k] = (uint16_t)t;
      }
      __syncwarp();
      if (k < n_rem) {
        const uint32_t f = P.patch[k];
        P.fn[f].w = INFINITY;
        P.fkey[f] = INFINITY;
      }
      if (on) {
        P.start_at[a] = kNoSlot;
        P.start_at[b] = kNoSlot;
      }
      __syncwarp();
      FCLG_EPA_PHASE(5);
      if (on) {
        write_face(t, a, b, vnew);
        P.fmark[t] = 0;
        P.fadj[t][0] = (uint16_t)g;
        const uint32_t gv = P.fv[g];
        int gj = -1;
#pragma unroll
        for (int h = 0; h < 3; ++h)
          if (fvert(gv, h) == b && fvert(gv, (h + 1) % 3) == a) gj = h;
        if (gj < 0) err = true;
        else P.fadj[g][gj] = (uint16_t)t;
        if (atomicCAS(&P.start_at[a], kNoSlot, t) != kNoSlot) err = true;
      }
      __syncwarp();
      if (on) {
        const uint32_t u = P.start_at[b];
        if (u == kNoSlot) {
          err = true;
        } else {
          P.fadj[t][1] = (uint16_t)u;
          P.fadj[u][2] = (uint16_t)t;
        }
      }
      __syncwarp();
      FCLG_EPA_PHASE(6);
      if (__any_sync(0xFFFFFFFFu, err)) return 2;
      live = new_live;
      fs_top = avail > n_hz ? avail - n_hz : 0;
      hw += fresh;
      return 0;
    }
    // Phase A: endpoints and outside neighbours of the horizon edges (the
    // patch slots are overwritten below); slots popped from the free stack.
    constexpr int kPer = (FMAX + 8 + 31) / 32;
    uint32_t ha[kPer], hb[kPer], hg[kPer];
    int j = 0;
    for (int k = (int)lane; k < n_hz; k += 32, ++j) {
      const uint32_t s = P.hz_s[k], e = P.hz_e[k];
      ha[j] = fvert(P.fv[s], (int)e);
      hb[j] = fvert(P.fv[s], (int)((e + 1) % 3));
      hg[j] = P.fadj[s][e];
      P.hz_slot[k] = (k < avail) ? P.freestk[avail - 1 - k] : (uint16_t)(hw + (k - avail));
    }
    __syncwarp();
    for (int k = (int)lane; k < n_rem; k += 32) {
      const uint32_t f = P.patch[k];
      P.fn[f].w = INFINITY;
      P.fkey[f] = INFINITY;
    }
    j = 0;
    for (int k = (int)lane; k < n_hz; k += 32, ++j) {
      P.start_at[ha[j]] = kNoSlot;
      P.start_at[hb[j]] = kNoSlot;
    }
    __syncwarp();
    FCLG_EPA_PHASE(5);
    // Phase B: write the fan (a, b, new) and re-point the outside neighbours.
    j = 0;
    for (int k = (int)lane; k < n_hz; k += 32, ++j) {
      const uint32_t t = P.hz_slot[k];
      const uint32_t a = ha[j], b = hb[j], g = hg[j];
      write_face(t, a, b, vnew);
      P.fmark[t] = 0;
      P.fadj[t][0] = (uint16_t)g;
      const uint32_t gv = P.fv[g];
      int gj = -1;
#pragma unroll
      for (int h = 0; h < 3; ++h)
        if (fvert(gv, h) == b && fvert(gv, (h + 1) % 3) == a) gj = h;
      if (gj < 0) err = true;
      else P.fadj[g][gj] = (uint16_t)t;
      if (atomicCAS(&P.start_at[a], kNoSlot, t) != kNoSlot) err = true;
    }
    __syncwarp();
    // Phase C: link consecutive fan faces.
    j = 0;
    for (int k = (int)lane; k < n_hz; k += 32, ++j) {
      const uint32_t t = P.hz_slot[k];
      const uint32_t u = P.start_at[hb[j]];
      if (u == kNoSlot) { err = true; continue; }
      P.fadj[t][1] = (uint16_t)u;
      P.fadj[u][2] = (uint16_t)t;
    }
    __syncwarp();
    FCLG_EPA_PHASE(6);
    if (__any_sync(0xFFFFFFFFu, err)) return 2;
    live = new_live;
    fs_top = avail > n_hz ? avail - n_hz : 0;
    hw += fresh;
    return 0;
  }

  // Writes the polytope state of a kEpaOverflow result (all lanes; layout
  // RF / RV = this layout's capacity).
  template <int RF, int RV>
  __device__ void save(unsigned char* rec, const EpaResult& r) const {
    using L = EpaResume<RF, RV>;
    static_assert(RF == FMAX && RV == VMAX, "a state is written in its own layout's sizes");
    if (lane == 0) {
      int* h = reinterpret_cast<int*>(rec + L::kHead);
      h[0] = r.resume_nv;
      h[1] = hw;
      h[2] = live;
      h[3] = fs_top;
      h[4] = r.iterations;
    }
    for (int i = (int)lane; i < hw; i += 32) {
      reinterpret_cast<float4*>(rec + L::kFn)[i] = P.fn[i];
      reinterpret_cast<float*>(rec + L::kFkey)[i] = P.fkey[i];
      reinterpret_cast<uint32_t*>(rec + L::kFv)[i] = P.fv[i];
      reinterpret_cast<uint2*>(rec + L::kFadj)[i] = *reinterpret_cast<const uint2*>(&P.fadj[i][0]);
    }
    for (int i = (int)lane; i < fs_top; i += 32) reinterpret_cast<uint16_t*>(rec + L::kFree)[i] = P.freestk[i];
    for (int i = (int)lane; i < r.resume_nv; i += 32) {
      reinterpret_cast<float4*>(rec + L::kVw)[i] = P.vw[i];
      reinterpret_cast<float4*>(rec + L::kVpa)[i] = P.vpa[i];
    }
  }

  // Continues a state written by a smaller layout (RF faces, RV vertices):
  // loads it and runs the remaining iterations.
  template <int RF, int RV>
  __device__ EpaResult resume(const unsigned char* rec, int max_iter, int max_faces, bool overflow_is_final) {
    using L = EpaResume<RF, RV>;
    static_assert(RF <= FMAX && RV <= VMAX, "a state continues in a layout at least as large");
    const int* h = reinterpret_cast<const int*>(rec + L::kHead);
    nv = h[0];
    hw = h[1];
    live = h[2];
    fs_top = h[3];
    const int it0 = h[4];
    for (int i = (int)lane; i < hw; i += 32) {
      P.fn[i] = reinterpret_cast<const float4*>(rec + L::kFn)[i];
      P.fkey[i] = reinterpret_cast<const float*>(rec + L::kFkey)[i];
      P.fv[i] = reinterpret_cast<const uint32_t*>(rec + L::kFv)[i];
      *reinterpret_cast<uint2*>(&P.fadj[i][0]) = reinterpret_cast<const uint2*>(rec + L::kFadj)[i];
      P.fmark[i] = 0;
    }
    for (int i = (int)lane; i < fs_top; i += 32) P.freestk[i] = reinterpret_cast<const uint16_t*>(rec + L::kFree)[i];
    for (int i = (int)lane; i < nv; i += 32) {
      P.vw[i] = reinterpret_cast<const float4*>(rec + L::kVw)[i];
      P.vpa[i] = reinterpret_cast<const float4*>(rec + L::kVpa)[i];
    }
    stamp = 0;
    __syncwarp();
    EpaResult r;
    r.status = kEpaFailed;
    r.depth = 0.f;
    r.p0 = r.p1 = mk3(0, 0, 0);
    r.iterations = it0;
    r.resume_nv = 0;
    r.fin_fv = kNoSlot;
    iterate(it0, max_iter, max_faces, overflow_is_final, r);
    return r;
  }

  // Runs EPA from the GJK simplex (rank, pa[], pb[]).  When this layout runs
  // out of face or vertex slots before max_faces, the result is kEpaOverflow
  // (continued or rerun in a larger layout) unless overflow_is_final.
  __device__ EpaResult run(int rank, const f3* spa, const f3* spb, int max_iter, int max_faces,
                           bool overflow_is_final) {
    EpaResult r;
    r.status = kEpaFailed;
    r.depth = 0.f;
    r.p0 = r.p1 = mk3(0, 0, 0);
    r.iterations = 0;
    r.resume_nv = 0;
    r.fin_fv = kNoSlot;
    nv = 0;
    hw = 0;
    live = 0;
    fs_top = 0;
    const float tol2 = tol * tol;
    for (int i = 0; i < rank; ++i) {
      if (sqn(spa[i] - spb[i]) <= tol2) { touching(spa[i], spb[i], r); return r; }
    }
    for (int i = 0; i < rank; ++i) push_vertex(spa[i], spb[i]);
    __syncwarp();
    bool done = false, ok = false;
    if (rank == 4) {
      const int faces[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 1, 3}, {1, 2, 3}};
      int tri = -1;
      for (int f = 0; f < 4 && tri < 0; ++f)
        if (point_to_plane(mk3(0, 0, 0), W(faces[f][0]), W(faces[f][1]), W(faces[f][2])) < tol) tri = f;
      if (tri < 0) {
        ok = tetra();
      } else {
        const f3 qa[3] = {spa[faces[tri][0]], spa[faces[tri][1]], spa[faces[tri][2]]};
        const f3 qb[3] = {spb[faces[tri][0]], spb[faces[tri][1]], spb[faces[tri][2]]};
        nv = 0;
        __syncwarp();
        for (int i = 0; i < 3; ++i) push_vertex(qa[i], qb[i]);
        __syncwarp();
        ok = from_triangle(r, done);
      }
    } else if (rank == 3) {
      ok = from_triangle(r, done);
    } else if (rank == 2) {
      ok = from_segment(r, done);
    } else {
      r.status = kEpaTouching;
      r.p0 = spa[0];
      r.p1 = spb[0];
      return r;
    }
    if (done) return r;
    if (!ok) { r.status = kEpaFailed; return r; }
    __syncwarp();
    iterate(0, max_iter, max_faces, overflow_is_final, r);
    return r;
  }

  // The expansion loop from iteration `it` on the current polytope.
  __device__ void iterate(int it, int max_iter, int max_faces, bool overflow_is_final, EpaResult& r) {
    for (;;) {
      int bs;
      float bd;
      FCLG_EPA_PHASE(0);
      nearest(bs, bd);
      FCLG_EPA_PHASE(1);
      if (bs == 0x7FFFFFFF || !(bd < INFINITY)) { r.status = kEpaFailed; return; }
      const f3 n = ld3(P.fn[bs]);
      const uint32_t bfv = P.fv[bs];  // the slot may be reused by the expansion below
      f3 pa, pb;
      sup(n, pa, pb);
      FCLG_EPA_PHASE(2);
      const float delta = dot(n, pa - pb) - bd;
      FCLG_EPA_TRACE(P, it, bs, bd, delta, live, hw, nv);
      if (delta <= tol) {
        finalize(bfv, pa, pb, r);
        r.status = kEpaOK;
        return;
      }
      if (nv >= VMAX) {
        finalize(bfv, pa, pb, r);
        r.status = overflow_is_final ? kEpaMallocFailed : kEpaOverflow;
        r.resume_nv = nv;  // the support is not in the polytope yet
        return;
      }
      push_vertex(pa, pb);
      __syncwarp();
      const int ex = expand(bs, max_faces);
      if (ex == 1 || (ex == 3 && overflow_is_final)) {
        finalize(bfv, pa, pb, r);
        r.status = kEpaMallocFailed;
        return;
      }
      if (ex == 3) {
        // the expansion stopped before changing the polytope: the state is
        // the one before this iteration, without the new vertex
        r.status = kEpaOverflow;
        r.resume_nv = nv - 1;
        return;
      }
      if (ex == 2) {
        // The visible patch has no simple horizon at FP32 resolution.  Near
        // convergence (support within 10 tolerances of the face) the current
        // nearest face is the answer; otherwise report failure.
        if (delta <= 10.f * tol) {
          finalize(bfv, pa, pb, r);
          r.status = kEpaOK;
        } else {
          r.status = kEpaFailed;
        }
        return;
      }
      ++it;
      r.iterations = it;
      if (it >= max_iter) {
        finalize(bfv, pa, pb, r);
        r.status = kEpaIterLimit;
        return;
      }
    }
  }
};

}  // namespace fclg
