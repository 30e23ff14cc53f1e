// Convex-hull vertex adjacency for the GPU support walk: quickhull in FP64
// (Barber, Dobkin and Huhdanpaa, 1996) over the hull's points, then each hull
// vertex's neighbours in the hull's edge graph.  fcl::Convex gets the same
// graph from the caller's face list (convex-inl.h:379-405, FindVertexNeighbors);
// the batch API takes vertices only, so the graph is rebuilt here once per shape.
#include "hull.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace fclg {
namespace {

struct P3 {
  double x, y, z;
};
inline P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dotp(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 crossp(P3 a, P3 b) { return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double len(P3 a) { return std::sqrt(dotp(a, a)); }

struct Face {
  int v[3];
  int adj[3];  // neighbour across edge k = (v[k], v[k+1])
  P3 n;        // outward unit normal
  double d;    // n . x = d on the plane
  bool alive;
  unsigned stamp;
  std::vector<int> conflict;
};

class Hull {
 public:
  Hull(const float* xyzw, uint32_t nv) : n_(nv) {
    p_.resize(nv);
    double extent = 0;
    for (uint32_t i = 0; i < nv; ++i) {
      p_[i] = P3{xyzw[4 * i], xyzw[4 * i + 1], xyzw[4 * i + 2]};
      extent = std::max({extent, std::fabs(p_[i].x), std::fabs(p_[i].y), std::fabs(p_[i].z)});
    }
    eps_ = 1e-7 * std::max(extent, 1e-30);
  }

  bool build() {
    int s[4];
    if (!initial(s)) return false;
    // tetrahedron faces, outward
    const int tf[4][3] = {{s[0], s[1], s[2]}, {s[0], s[2], s[3]}, {s[0], s[3], s[1]}, {s[1], s[3], s[2]}};
    P3 c{0, 0, 0};
    for (int i = 0; i < 4; ++i) c = P3{c.x + p_[s[i]].x / 4, c.y + p_[s[i]].y / 4, c.z + p_[s[i]].z / 4};
    for (int i = 0; i < 4; ++i) {
      int a = tf[i][0], b = tf[i][1], cc = tf[i][2];
      Face f = make_face(a, b, cc);
      if (dotp(f.n, c) - f.d > 0) f = make_face(a, cc, b);
      faces_.push_back(f);
    }
    link_all_initial();
    std::vector<char> used(n_, 0);
    for (int i = 0; i < 4; ++i) used[s[i]] = 1;
    for (uint32_t i = 0; i < n_; ++i)
      if (!used[i]) assign((int)i, 0, 4);
    // expand: faces holding outside points, the new faces pushed as they appear
    std::vector<int> work;
    for (int i = 0; i < 4; ++i)
      if (!faces_[i].conflict.empty()) work.push_back(i);
    while (!work.empty()) {
      const int fi = work.back();
      work.pop_back();
      if (!faces_[fi].alive || faces_[fi].conflict.empty()) continue;
      const size_t first = faces_.size();
      if (!add_point(fi)) return false;
      for (size_t i = first; i < faces_.size(); ++i)
        if (!faces_[i].conflict.empty()) work.push_back((int)i);
    }
    return true;
  }

  void graph(HullGraph& g) const {
    std::vector<std::vector<uint32_t>> rows(n_);
    for (const Face& f : faces_) {
      if (!f.alive) continue;
      for (int k = 0; k < 3; ++k) rows[f.v[k]].push_back((uint32_t)f.v[(k + 1) % 3]);
    }
    // six axis extremes over the hull's corners (first index on ties)
    const P3 axes[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int a = 0; a < 6; ++a) {
      int best = -1;
      double bv = 0;
      for (uint32_t i = 0; i < n_; ++i) {
        if (rows[i].empty()) continue;
        const double v = dotp(axes[a], p_[i]);
        if (best < 0 || v > bv) { best = (int)i; bv = v; }
      }
      g.start[a] = (uint32_t)best;
    }
    // rows ascending, as the reference's per-vertex std::set
    g.first.assign(n_ + 1, 0);
    g.adj.clear();
    for (uint32_t i = 0; i < n_; ++i) {
      std::sort(rows[i].begin(), rows[i].end());
      g.first[i] = (uint32_t)g.adj.size();
      g.adj.insert(g.adj.end(), rows[i].begin(), rows[i].end());
    }
    g.first[n_] = (uint32_t)g.adj.size();
  }

 private:
  uint32_t n_;
  std::vector<P3> p_;
  double eps_;
  std::vector<Face> faces_;
  unsigned stamp_ = 0;

  double dist(const Face& f, int i) const { return dotp(f.n, p_[i]) - f.d; }

  Face make_face(int a, int b, int c) const {
    Face f;
    f.v[0] = a;
    f.v[1] = b;
    f.v[2] = c;
    f.adj[0] = f.adj[1] = f.adj[2] = -1;
    P3 n = crossp(sub(p_[b], p_[a]), sub(p_[c], p_[a]));
    const double l = len(n);
    f.n = l > 0 ? P3{n.x / l, n.y / l, n.z / l} : P3{0, 0, 0};
    f.d = dotp(f.n, p_[a]);
    f.alive = true;
    f.stamp = 0;
    return f;
  }

  bool initial(int s[4]) {
    if (n_ < 4) return false;
    // the farthest pair among the six axis extremes
    int ext[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = 1; i < n_; ++i) {
      if (p_[i].x < p_[ext[0]].x) ext[0] = (int)i;
      if (p_[i].x > p_[ext[1]].x) ext[1] = (int)i;
      if (p_[i].y < p_[ext[2]].y) ext[2] = (int)i;
      if (p_[i].y > p_[ext[3]].y) ext[3] = (int)i;
      if (p_[i].z < p_[ext[4]].z) ext[4] = (int)i;
      if (p_[i].z > p_[ext[5]].z) ext[5] = (int)i;
    }
    double best = -1;
    for (int a = 0; a < 6; ++a)
      for (int b = a + 1; b < 6; ++b) {
        const double d = len(sub(p_[ext[a]], p_[ext[b]]));
        if (d > best) { best = d; s[0] = ext[a]; s[1] = ext[b]; }
      }
    if (best <= eps_) return false;
    const P3 u = sub(p_[s[1]], p_[s[0]]);
    best = -1;
    for (uint32_t i = 0; i < n_; ++i) {
      const double d = len(crossp(u, sub(p_[i], p_[s[0]])));
      if (d > best) { best = d; s[2] = (int)i; }
    }
    if (best <= eps_ * len(u)) return false;
    const P3 n = crossp(u, sub(p_[s[2]], p_[s[0]]));
    const double nl = len(n);
    best = -1;
    for (uint32_t i = 0; i < n_; ++i) {
      const double d = std::fabs(dotp(n, sub(p_[i], p_[s[0]]))) / nl;
      if (d > best) { best = d; s[3] = (int)i; }
    }
    return best > eps_;
  }

  // edge (a, b) of face f -> index k with v[k] = a, v[k+1] = b, or -1
  static int edge_index(const Face& f, int a, int b) {
    for (int k = 0; k < 3; ++k)
      if (f.v[k] == a && f.v[(k + 1) % 3] == b) return k;
    return -1;
  }

  void link_all_initial() {
    for (int i = 0; i < 4; ++i)
      for (int k = 0; k < 3; ++k) {
        const int a = faces_[i].v[k], b = faces_[i].v[(k + 1) % 3];
        for (int j = 0; j < 4; ++j) {
          if (j == i) continue;
          if (edge_index(faces_[j], b, a) >= 0) faces_[i].adj[k] = j;
        }
      }
  }

  void assign(int pt, size_t f_begin, size_t f_end) {
    for (size_t f = f_begin; f < f_end; ++f) {
      if (!faces_[f].alive) continue;
      if (dist(faces_[f], pt) > eps_) {
        faces_[f].conflict.push_back(pt);
        return;
      }
    }
  }

  bool add_point(int fi) {
    // farthest conflict point of the face
    const Face& f0 = faces_[fi];
    int p = f0.conflict[0];
    double pd = dist(f0, p);
    for (int q : f0.conflict) {
      const double d = dist(f0, q);
      if (d > pd) { pd = d; p = q; }
    }
    // visible faces (flood fill from fi)
    ++stamp_;
    std::vector<int> visible{fi}, stack{fi};
    faces_[fi].stamp = stamp_;
    while (!stack.empty()) {
      const int g = stack.back();
      stack.pop_back();
      for (int k = 0; k < 3; ++k) {
        const int h = faces_[g].adj[k];
        if (h < 0) return false;
        if (faces_[h].stamp == stamp_) continue;
        if (dist(faces_[h], p) > eps_) {
          faces_[h].stamp = stamp_;
          visible.push_back(h);
          stack.push_back(h);
        }
      }
    }
    // horizon edges: (a, b) of a visible face whose neighbour is not visible
    struct Hz {
      int a, b, outside;
    };
    std::vector<Hz> hz;
    for (int g : visible)
      for (int k = 0; k < 3; ++k) {
        const int h = faces_[g].adj[k];
        if (faces_[h].stamp != stamp_) hz.push_back(Hz{faces_[g].v[k], faces_[g].v[(k + 1) % 3], h});
      }
    if (hz.size() < 3) return false;
    // new faces (a, b, p), linked through the horizon's start / end vertices
    std::vector<int> start_at(n_, -1), end_at(n_, -1);
    const size_t first = faces_.size();
    for (const Hz& e : hz) {
      const int nf = (int)faces_.size();
      faces_.push_back(make_face(e.a, e.b, p));
      faces_.back().adj[0] = e.outside;
      const int k = edge_index(faces_[e.outside], e.b, e.a);
      if (k < 0) return false;
      faces_[e.outside].adj[k] = nf;
      if (start_at[e.a] >= 0 || end_at[e.b] >= 0) return false;  // not a simple horizon
      start_at[e.a] = nf;
      end_at[e.b] = nf;
    }
    for (size_t i = first; i < faces_.size(); ++i) {
      Face& nf = faces_[i];
      nf.adj[1] = start_at[nf.v[1]];  // edge (b, p): the new face whose horizon edge starts at b
      nf.adj[2] = end_at[nf.v[0]];    // edge (p, a): the new face whose horizon edge ends at a
      if (nf.adj[1] < 0 || nf.adj[2] < 0) return false;
    }
    // retire the visible faces and hand their points to the new ones
    std::vector<int> orphans;
    for (int g : visible) {
      faces_[g].alive = false;
      for (int q : faces_[g].conflict)
        if (q != p) orphans.push_back(q);
      faces_[g].conflict.clear();
      faces_[g].conflict.shrink_to_fit();
    }
    for (int q : orphans) assign(q, first, faces_.size());
    return true;
  }
};

}  // namespace

bool hull_graph(const float* xyzw, uint32_t nv, HullGraph& g) {
  g.first.clear();
  g.adj.clear();
  if (nv < 4) return false;
  Hull h(xyzw, nv);
  if (!h.build()) return false;
  h.graph(g);
  return true;
}

bool pack_walk(const float* xyzw, const HullGraph& g, std::vector<float>& out) {
  const uint32_t nv = (uint32_t)g.first.size() - 1;
  // entry of each hull vertex's row: 6 start entries come first
  std::vector<uint32_t> link(nv, 0);
  uint32_t row = 6;
  for (uint32_t i = 0; i < nv; ++i) {
    const uint32_t deg = g.first[i + 1] - g.first[i];
    if (deg == 0) continue;
    if (deg > kWalkMaxDegree || row >= (1u << 24)) return false;
    link[i] = (row << 8) | deg;
    row += deg;
  }
  const size_t base = out.size();
  out.resize(base + 4 * (size_t)row);
  float* e = out.data() + base;
  auto put = [&](size_t k, uint32_t v) {
    e[4 * k] = xyzw[4 * v];
    e[4 * k + 1] = xyzw[4 * v + 1];
    e[4 * k + 2] = xyzw[4 * v + 2];
    std::memcpy(&e[4 * k + 3], &link[v], sizeof(uint32_t));
  };
  for (int a = 0; a < 6; ++a) put(a, g.start[a]);
  size_t k = 6;
  for (uint32_t i = 0; i < nv; ++i)
    for (uint32_t j = g.first[i]; j < g.first[i + 1]; ++j) put(k++, g.adj[j]);
  return true;
}

}  // namespace fclg
