// Adaptive mesh refinement, host side, native: the block tree, the neighbour lists and
// coordinates of every block, the refinement flags and the tree update — what the
// reference's Mesh does on the host between two cycles (mesh/meshblock_tree.cpp,
// bvals/bvals_base.cpp:300-720, mesh/mesh.cpp:1984-2060, mesh/mesh_refinement.cpp:
// 1393-1455, mesh/amr_loadbalance.cpp:178-317 and the maps of :351-660).  Host-only code;
// athgpu_amr_step runs a whole refinement check and regrid with no Python in between.
// The Python restatement in athena_gb300/meshtree.py and athena_gb300/amr.py is the
// checker of this file (tests/test_amr_native.py compares every table).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/athena_gb300.h"

namespace athgpu {
athgpu_status api_fail(athgpu_status code, const std::string& msg);
}

namespace {
using athgpu::api_fail;

struct Loc {
  int level;
  long long lx[3];
  bool operator<(const Loc& o) const {
    return std::tie(level, lx[0], lx[1], lx[2]) < std::tie(o.level, o.lx[0], o.lx[1], o.lx[2]);
  }
  bool operator==(const Loc& o) const {
    return level == o.level && lx[0] == o.lx[0] && lx[1] == o.lx[1] && lx[2] == o.lx[2];
  }
};

Loc child_loc(const Loc& p, int i, int j, int k) {
  return Loc{p.level + 1, {2 * p.lx[0] + i, 2 * p.lx[1] + j, 2 * p.lx[2] + k}};
}

// MeshBlockTree (mesh/meshblock_tree.cpp): nodes in a pool, children by index
class BlockTree {
 public:
  struct Node {
    Loc loc;
    int leaf[8];
    bool refined;
    int gid;
  };
  int nrbx[3], bcs[6], root_level = 0;
  long long nnew = 0, ndel = 0;
  std::vector<Node> nodes;
  std::vector<int> free_nodes;

  BlockTree(const int nr[3], const int bc[6]) {
    for (int d = 0; d < 3; ++d) nrbx[d] = nr[d];
    for (int f = 0; f < 6; ++f) bcs[f] = bc[f];
    const int nbmax = std::max(nrbx[0], std::max(nrbx[1], nrbx[2]));
    while ((1 << root_level) < nbmax) ++root_level;
    const int r = make(Loc{0, {0, 0, 0}}, -1);
    create_root(r);
  }
  int make(const Loc& l, int gid) {
    Node n;
    n.loc = l;
    for (int q = 0; q < 8; ++q) n.leaf[q] = -1;
    n.refined = false;
    n.gid = gid;
    if (!free_nodes.empty()) {
      const int i = free_nodes.back();
      free_nodes.pop_back();
      nodes[i] = n;
      return i;
    }
    nodes.push_back(n);
    return (int)nodes.size() - 1;
  }
  // the root grid (meshblock_tree.cpp:87-132)
  void create_root(int nd) {
    const Loc l = nodes[nd].loc;
    if (l.level == root_level) return;
    nodes[nd].refined = true;
    const long long levfac = 1LL << (root_level - l.level - 1);
    for (int n = 0; n < 8; ++n) {
      const int i = n & 1, j = (n >> 1) & 1, k = (n >> 2) & 1;
      if ((l.lx[2] * 2 + k) * levfac < nrbx[2] && (l.lx[1] * 2 + j) * levfac < nrbx[1] &&
          (l.lx[0] * 2 + i) * levfac < nrbx[0]) {
        const int c = make(child_loc(l, i, j, k), -1);
        nodes[nd].leaf[n] = c;
        create_root(c);
      }
    }
  }
  long long nblocks_at(int d, int level) const { return (long long)nrbx[d] << (level - root_level); }
  // AddMeshBlock: make rloc a leaf, refining on the way
  void add(int nd, const Loc& r) {
    if (nodes[nd].loc.level == r.level) return;
    if (!nodes[nd].refined) refine(nd);
    const int sh = r.level - nodes[nd].loc.level - 1;
    const int n = (int)(((r.lx[0] >> sh) & 1) + (((r.lx[1] >> sh) & 1) << 1) +
                        (((r.lx[2] >> sh) & 1) << 2));
    add(nodes[nd].leaf[n], r);
  }
  // Refine (meshblock_tree.cpp:166-258): split a leaf; the children inherit its gid; every
  // neighbour at the leaf's level becomes a leaf or finer
  void refine(int nd) {
    if (nodes[nd].refined) return;
    nnew += 7;
    const Loc l = nodes[nd].loc;
    const int gid = nodes[nd].gid;
    for (int n = 0; n < 8; ++n) {
      const int c = make(child_loc(l, n & 1, (n >> 1) & 1, (n >> 2) & 1), gid);
      nodes[nd].leaf[n] = c;
    }
    nodes[nd].refined = true;
    const long long nmax[3] = {nblocks_at(0, l.level), nblocks_at(1, l.level),
                               nblocks_at(2, l.level)};
    for (int oz = -1; oz <= 1; ++oz) {
      long long lz = l.lx[2] + oz;
      if (lz < 0) { if (bcs[4] != 0) continue; lz = nmax[2] - 1; }
      if (lz >= nmax[2]) { if (bcs[5] != 0) continue; lz = 0; }
      for (int oy = -1; oy <= 1; ++oy) {
        long long ly = l.lx[1] + oy;
        if (ly < 0) { if (bcs[2] != 0) continue; ly = nmax[1] - 1; }
        if (ly >= nmax[1]) { if (bcs[3] != 0) continue; ly = 0; }
        for (int ox = -1; ox <= 1; ++ox) {
          if (ox == 0 && oy == 0 && oz == 0) continue;
          long long lx = l.lx[0] + ox;
          if (lx < 0) { if (bcs[0] != 0) continue; lx = nmax[0] - 1; }
          if (lx >= nmax[0]) { if (bcs[1] != 0) continue; lx = 0; }
          add(0, Loc{l.level, {lx, ly, lz}});
        }
      }
    }
    nodes[nd].gid = -1;
  }
  void release(int nd) {
    if (nodes[nd].refined)
      for (int n = 0; n < 8; ++n)
        if (nodes[nd].leaf[n] >= 0) release(nodes[nd].leaf[n]);
    free_nodes.push_back(nd);
  }
  // Derefine's test (meshblock_tree.cpp:261-303)
  bool derefine_ok(int nd) const {
    const Loc l = nodes[nd].loc;
    for (int ox3 = -1; ox3 <= 1; ++ox3)
      for (int ox2 = -1; ox2 <= 1; ++ox2)
        for (int ox1 = -1; ox1 <= 1; ++ox1) {
          const int bt = find_neighbor(l, ox1, ox2, ox3, true);
          if (bt < 0 || !nodes[bt].refined) continue;
          const int o[3] = {ox1, ox2, ox3};
          int lo[3], hi[3];
          for (int a = 0; a < 3; ++a) {
            lo[a] = o[a] == -1 ? 1 : 0;
            hi[a] = o[a] == 1 ? 0 : 1;
          }
          for (int lk = lo[2]; lk <= hi[2]; ++lk)
            for (int lj = lo[1]; lj <= hi[1]; ++lj)
              for (int li = lo[0]; li <= hi[0]; ++li) {
                const int c = nodes[bt].leaf[li + (lj << 1) + (lk << 2)];
                if (c >= 0 && nodes[c].refined) return false;
              }
        }
    return true;
  }
  void derefine(int nd) {
    nodes[nd].gid = nodes[nodes[nd].leaf[0]].gid;
    for (int n = 0; n < 8; ++n)
      if (nodes[nd].leaf[n] >= 0) release(nodes[nd].leaf[n]);
    for (int n = 0; n < 8; ++n) nodes[nd].leaf[n] = -1;
    nodes[nd].refined = false;
    ndel += 7;
  }
  // leaves in gid order; old[] receives each leaf's previous gid (GetMeshBlockList)
  void block_list(std::vector<Loc>* out, std::vector<int>* old) {
    out->clear();
    if (old) old->clear();
    walk(0, out, old);
  }
  void walk(int nd, std::vector<Loc>* out, std::vector<int>* old) {
    if (!nodes[nd].refined) {
      if (old) old->push_back(nodes[nd].gid);
      nodes[nd].gid = (int)out->size();
      out->push_back(nodes[nd].loc);
      return;
    }
    for (int n = 0; n < 8; ++n)
      if (nodes[nd].leaf[n] >= 0) walk(nodes[nd].leaf[n], out, old);
  }
  int find(const Loc& l) const {
    int nd = 0;
    while (nodes[nd].loc.level != l.level) {
      if (!nodes[nd].refined) return -1;
      const int sh = l.level - nodes[nd].loc.level - 1;
      const int n = (int)(((l.lx[0] >> sh) & 1) + (((l.lx[1] >> sh) & 1) << 1) +
                          (((l.lx[2] >> sh) & 1) << 2));
      nd = nodes[nd].leaf[n];
      if (nd < 0) return -1;
    }
    return nd;
  }
  // FindNeighbor (meshblock_tree.cpp:362-420): the leaf at the same or a coarser level,
  // or the refined node whose children are the finer neighbours; -1 across a physical
  // mesh face; -2 if the tree is broken
  int find_neighbor(const Loc& loc, int ox1, int ox2, int ox3, bool amrflag) const {
    const int ll = loc.level;
    long long l[3] = {loc.lx[0] + ox1, loc.lx[1] + ox2, loc.lx[2] + ox3};
    for (int d = 0; d < 3; ++d) {
      const long long n = nblocks_at(d, ll);
      if (l[d] < 0) { if (bcs[2 * d] != 0) return -1; l[d] = n - 1; }
      if (l[d] >= n) { if (bcs[2 * d + 1] != 0) return -1; l[d] = 0; }
    }
    if (ll < 1) return 0;
    int bt = 0;
    for (int level = 0; level < ll; ++level) {
      if (!nodes[bt].refined) {
        if (level == ll - 1) return bt;
        return -2;
      }
      const int sh = ll - level - 1;
      bt = nodes[bt].leaf[((l[0] >> sh) & 1) + (((l[1] >> sh) & 1) << 1) +
                          (((l[2] >> sh) & 1) << 2)];
      if (bt < 0) return -2;
    }
    if (!nodes[bt].refined) return bt;
    const int fl = nodes[bt].leaf[(ox1 < 0 ? 1 : 0) + ((ox2 < 0 ? 1 : 0) << 1) +
                                  ((ox3 < 0 ? 1 : 0) << 2)];
    if (!nodes[fl].refined || amrflag) return bt;
    return -2;
  }
  int child(int nd, int i, int j, int k) const { return nodes[nd].leaf[i + (j << 1) + (k << 2)]; }
};

enum { NF = 10, MAXNB = 56 };

// BoundaryBase::SearchAndSetNeighbors (bvals/bvals_base.cpp:300-720), 3-D: the neighbour
// entries (gid, level, ox1, ox2, ox3, type, fi1, fi2, fid, eid) in the reference's order
// and nblevel[(ox3+1)*9 + (ox2+1)*3 + (ox1+1)]; false if the tree is broken
bool neighbors(const BlockTree& t, const Loc& loc, int* table, int* count, int* nblevel) {
  for (int q = 0; q < 27; ++q) nblevel[q] = -1;
  nblevel[13] = loc.level;
  int myox[3];
  for (int a = 0; a < 3; ++a) myox[a] = 2 * (int)(loc.lx[a] & 1) - 1;
  int nn = 0;
  auto push = [&](int gid, int level, int o1, int o2, int o3, int type, int f1, int f2,
                  int fid, int eid) {
    if (nn >= MAXNB) return false;
    int* e = table + nn * NF;
    e[0] = gid; e[1] = level; e[2] = o1; e[3] = o2; e[4] = o3; e[5] = type;
    e[6] = f1; e[7] = f2; e[8] = fid; e[9] = eid;
    ++nn;
    return true;
  };
  auto lv = [&](int o1, int o2, int o3) -> int& {
    return nblevel[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
  };
  // faces
  for (int d = 0; d < 3; ++d)
    for (int n = -1; n <= 1; n += 2) {
      int o[3] = {0, 0, 0};
      o[d] = n;
      const int bt = t.find_neighbor(loc, o[0], o[1], o[2], false);
      if (bt == -2) return false;
      if (bt < 0) continue;
      const int fid = 2 * d + (n > 0 ? 1 : 0);
      const BlockTree::Node& B = t.nodes[bt];
      if (B.refined) {
        lv(o[0], o[1], o[2]) = B.loc.level + 1;
        const int fface = 1 - (n + 1) / 2;
        for (int f2 = 0; f2 <= 1; ++f2)
          for (int f1 = 0; f1 <= 1; ++f1) {
            int c[3];
            int q = 0;
            for (int a = 0; a < 3; ++a) c[a] = (a == d) ? fface : (q++ == 0 ? f1 : f2);
            const BlockTree::Node& L = t.nodes[t.child(bt, c[0], c[1], c[2])];
            if (!push(L.gid, L.loc.level, o[0], o[1], o[2], 0, f1, f2, fid, -1)) return false;
          }
      } else {
        lv(o[0], o[1], o[2]) = B.loc.level;
        if (!push(B.gid, B.loc.level, o[0], o[1], o[2], 0, 0, 0, fid, -1)) return false;
      }
    }
  // edges x1x2 (o3 = 0), x1x3 (o2 = 0), x2x3 (o1 = 0); outer loop over the second axis
  const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int p = 0; p < 3; ++p) {
    const int a = pairs[p][0], b = pairs[p][1];
    for (int m = -1; m <= 1; m += 2)
      for (int n = -1; n <= 1; n += 2) {
        int o[3] = {0, 0, 0};
        o[a] = n;
        o[b] = m;
        const int bt = t.find_neighbor(loc, o[0], o[1], o[2], false);
        if (bt == -2) return false;
        if (bt < 0) continue;
        const int eid = 4 * p + (((n + 1) >> 1) | ((m + 1) & 2));
        const BlockTree::Node& B = t.nodes[bt];
        if (B.refined) {
          lv(o[0], o[1], o[2]) = B.loc.level + 1;
          const int ff1 = 1 - (n + 1) / 2, ff2 = 1 - (m + 1) / 2;
          for (int f1 = 0; f1 <= 1; ++f1) {
            int c[3];
            c[a] = ff1;
            c[b] = ff2;
            c[3 - a - b] = f1;
            const BlockTree::Node& L = t.nodes[t.child(bt, c[0], c[1], c[2])];
            if (!push(L.gid, L.loc.level, o[0], o[1], o[2], 1, f1, 0, -1, eid)) return false;
          }
        } else {
          lv(o[0], o[1], o[2]) = B.loc.level;
          if (B.loc.level >= loc.level || (myox[a] == n && myox[b] == m))
            if (!push(B.gid, B.loc.level, o[0], o[1], o[2], 1, 0, 0, -1, eid)) return false;
        }
      }
  }
  // corners
  for (int l = -1; l <= 1; l += 2)
    for (int m = -1; m <= 1; m += 2)
      for (int n = -1; n <= 1; n += 2) {
        int bt = t.find_neighbor(loc, n, m, l, false);
        if (bt == -2) return false;
        if (bt < 0) continue;
        if (t.nodes[bt].refined)
          bt = t.child(bt, 1 - (n + 1) / 2, 1 - (m + 1) / 2, 1 - (l + 1) / 2);
        const BlockTree::Node& B = t.nodes[bt];
        lv(n, m, l) = B.loc.level;
        if (B.loc.level >= loc.level || (myox[0] == n && myox[1] == m && myox[2] == l))
          if (!push(B.gid, B.loc.level, n, m, l, 2, 0, 0, -1, -1)) return false;
      }
  *count = nn;
  return true;
}

// ComputeMeshGeneratorX with sym_interval (mesh.hpp:457-472) and UniformMeshGeneratorX
// (mesh.hpp:535-553)
double gen_x(long long index, long long nrange) {
  const long long noffset = index - nrange / 2;
  const long long noffset_ceil = index - (nrange + 1) / 2;
  return (double)(noffset + noffset_ceil) / (2.0 * (double)nrange);
}
double uniform_gen(double x, double xmin, double xmax) {
  return 0.5 * (xmin + xmax) + (x * xmax - x * xmin);
}

struct MeshGeom {
  int nx[3], nrbx[3], bx[3], ng, bcs[6];
  double xmin[3], xmax[3];
};

// block_size bounds (Mesh::SetBlockSizeAndBoundaries, mesh.cpp:1984-2060) and the face
// coordinates of a block (coarse: the coarse buffer's), with the reflecting-boundary
// ghost spacing (coordinates.cpp:92-161)
void block_faces(const MeshGeom& g, int root_level, const Loc& l, int d, bool coarse,
                 double* xf, double* dxf) {
  const int n = g.bx[d], ng = g.ng;
  const int nint = coarse ? n / 2 : n;
  const int nc = nint + 2 * ng;
  const int il = ng, iu = ng + nint - 1;
  const long long lx = l.lx[d];
  const long long nblev = (long long)g.nrbx[d] << (l.level - root_level);
  const double lo = lx == 0 ? g.xmin[d] : uniform_gen(gen_x(lx, nblev), g.xmin[d], g.xmax[d]);
  const double hi = lx == nblev - 1 ? g.xmax[d]
                                    : uniform_gen(gen_x(lx + 1, nblev), g.xmin[d], g.xmax[d]);
  const long long nroot = (long long)g.nx[d] << (l.level - root_level);
  for (int i = 0; i <= nc; ++i) {
    const long long off = coarse ? (long long)(i - il) * 2 + lx * n : (long long)(i - il) + lx * n;
    xf[i] = uniform_gen(gen_x(off, nroot), g.xmin[d], g.xmax[d]);
  }
  xf[il] = lo;
  xf[iu + 1] = hi;
  const double dx = (hi - lo) / (double)(iu - il + 1);
  for (int i = 0; i < nc; ++i) dxf[i] = dx;
  if (lx == 0 && g.bcs[2 * d] == ATHGPU_BC_REFLECT)
    for (int q = 1; q <= ng; ++q) {
      dxf[il - q] = dxf[il + q - 1];
      xf[il - q] = xf[il - q + 1] - dxf[il - q];
    }
  if (lx == nblev - 1 && g.bcs[2 * d + 1] == ATHGPU_BC_REFLECT)
    for (int q = 1; q <= ng; ++q) {
      dxf[iu + q] = dxf[iu - q + 1];
      xf[iu + q + 1] = xf[iu + q] + dxf[iu + q];
    }
}

}  // namespace

// ---- the adaptive mesh object ------------------------------------------------------------
struct athgpu_amr {
  MeshGeom g;
  BlockTree tree;
  int max_level, derefine_count;
  std::vector<Loc> locs;
  std::vector<int> deref;       // MeshRefinement::deref_count_ per block
  std::vector<int> table, count, nblevel;
  // the pending regrid (athgpu_amr_update)
  bool pending = false;
  std::vector<Loc> new_locs;
  std::vector<int> newtoold, kind, ffc, new_deref;
  athgpu_amr(const MeshGeom& geom, const int nr[3], const int bc[6])
      : g(geom), tree(nr, bc) {}

  bool rebuild_tables(const std::vector<Loc>& L, std::vector<int>* t, std::vector<int>* c,
                      std::vector<int>* nl) const {
    const size_t nb = L.size();
    t->assign(nb * MAXNB * NF, -1);
    c->assign(nb, 0);
    nl->assign(nb * 27, -1);
    for (size_t b = 0; b < nb; ++b)
      if (!neighbors(tree, L[b], t->data() + b * MAXNB * NF, c->data() + b, nl->data() + b * 27))
        return false;
    return true;
  }
};

namespace {
athgpu_status fill_tables(const athgpu_amr* a, long long* loc, int* nbr_table, int* nbr_count,
                          int* nblevel, double* const fine[6], double* const coarse[6]) {
  const size_t nb = a->locs.size();
  if (loc)
    for (size_t b = 0; b < nb; ++b) {
      loc[b * 4] = a->locs[b].level;
      for (int d = 0; d < 3; ++d) loc[b * 4 + 1 + d] = a->locs[b].lx[d];
    }
  if (nbr_table) std::memcpy(nbr_table, a->table.data(), sizeof(int) * a->table.size());
  if (nbr_count) std::memcpy(nbr_count, a->count.data(), sizeof(int) * a->count.size());
  if (nblevel) std::memcpy(nblevel, a->nblevel.data(), sizeof(int) * a->nblevel.size());
  for (int d = 0; d < 3; ++d) {
    const int nc = a->g.bx[d] + 2 * a->g.ng, ncc = a->g.bx[d] / 2 + 2 * a->g.ng;
    std::vector<double> xf(nc + 1), dxf(nc);
    for (size_t b = 0; b < nb; ++b) {
      if (fine[2 * d] || fine[2 * d + 1]) {
        block_faces(a->g, a->tree.root_level, a->locs[b], d, false, xf.data(), dxf.data());
        if (fine[2 * d]) std::memcpy(fine[2 * d] + b * (nc + 1), xf.data(), sizeof(double) * (nc + 1));
        if (fine[2 * d + 1]) std::memcpy(fine[2 * d + 1] + b * nc, dxf.data(), sizeof(double) * nc);
      }
      if (coarse[2 * d] || coarse[2 * d + 1]) {
        block_faces(a->g, a->tree.root_level, a->locs[b], d, true, xf.data(), dxf.data());
        if (coarse[2 * d]) std::memcpy(coarse[2 * d] + b * (ncc + 1), xf.data(), sizeof(double) * (ncc + 1));
        if (coarse[2 * d + 1]) std::memcpy(coarse[2 * d + 1] + b * ncc, dxf.data(), sizeof(double) * ncc);
      }
    }
  }
  return ATHGPU_OK;
}
}  // namespace

athgpu_status athgpu_amr_create(athgpu_amr** out, const int* nx, const int* nrbx, int nghost,
                                const double* xmin, const double* xmax, const int* bc,
                                int numlevel, int derefine_count) {
  if (!out || !nx || !nrbx || !xmin || !xmax || !bc) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *out = nullptr;
  MeshGeom g;
  for (int d = 0; d < 3; ++d) {
    if (nrbx[d] < 1 || nx[d] < 1 || nx[d] % nrbx[d])
      return api_fail(ATHGPU_ERR_ARG, "mesh size not divisible by the root grid");
    g.nx[d] = nx[d];
    g.nrbx[d] = nrbx[d];
    g.bx[d] = nx[d] / nrbx[d];
    if (g.bx[d] % 2 || g.bx[d] < 4)
      return api_fail(ATHGPU_ERR_ARG, "MeshBlock sizes must be even and at least 4");
    g.xmin[d] = xmin[d];
    g.xmax[d] = xmax[d];
  }
  if (nghost < 2 || nghost % 2) return api_fail(ATHGPU_ERR_ARG, "nghost must be even");
  if (numlevel < 1) return api_fail(ATHGPU_ERR_ARG, "numlevel must be at least 1");
  g.ng = nghost;
  for (int f = 0; f < 6; ++f) g.bcs[f] = bc[f];
  athgpu_amr* a = new athgpu_amr(g, nrbx, bc);
  a->max_level = a->tree.root_level + numlevel - 1;   // mesh.cpp:323
  a->derefine_count = derefine_count;
  a->tree.block_list(&a->locs, nullptr);
  a->deref.assign(a->locs.size(), 0);
  if (!a->rebuild_tables(a->locs, &a->table, &a->count, &a->nblevel)) {
    delete a;
    return api_fail(ATHGPU_ERR_ARG, "neighbour search failed");
  }
  *out = a;
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_destroy(athgpu_amr* a) {
  delete a;
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_add_block(athgpu_amr* a, int level, long long lx1, long long lx2,
                                   long long lx3) {
  if (!a) return api_fail(ATHGPU_ERR_ARG, "null argument");
  if (level < a->tree.root_level || level > a->max_level)
    return api_fail(ATHGPU_ERR_ARG, "level outside [root, root + numlevel - 1]");
  const long long l[3] = {lx1, lx2, lx3};
  for (int d = 0; d < 3; ++d)
    if (l[d] < 0 || l[d] >= a->tree.nblocks_at(d, level))
      return api_fail(ATHGPU_ERR_ARG, "logical location outside the mesh");
  a->tree.add(0, Loc{level, {lx1, lx2, lx3}});
  a->tree.block_list(&a->locs, nullptr);
  a->deref.assign(a->locs.size(), 0);
  if (!a->rebuild_tables(a->locs, &a->table, &a->count, &a->nblevel))
    return api_fail(ATHGPU_ERR_ARG, "neighbour search failed");
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_nblocks(const athgpu_amr* a, int* nb) {
  if (!a || !nb) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *nb = (int)a->locs.size();
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_tables(const athgpu_amr* a, long long* loc, int* nbr_table,
                                int* nbr_count, int* nblevel, double* x1f, double* dx1f,
                                double* x2f, double* dx2f, double* x3f, double* dx3f,
                                double* cx1f, double* cdx1f, double* cx2f, double* cdx2f,
                                double* cx3f, double* cdx3f) {
  if (!a) return api_fail(ATHGPU_ERR_ARG, "null argument");
  double* const fine[6] = {x1f, dx1f, x2f, dx2f, x3f, dx3f};
  double* const coarse[6] = {cx1f, cdx1f, cx2f, cdx2f, cx3f, cdx3f};
  return fill_tables(a, loc, nbr_table, nbr_count, nblevel, fine, coarse);
}

athgpu_status athgpu_amr_flags(athgpu_amr* a, const int* ret, int* flags) {
  if (!a || !ret || !flags) return api_fail(ATHGPU_ERR_ARG, "null argument");
  const int root = a->tree.root_level;
  for (size_t b = 0; b < a->locs.size(); ++b) {
    // MeshRefinement::CheckRefinementCondition (mesh_refinement.cpp:1393-1455)
    const int aret = std::max(-1, ret[b]);
    const int level = a->locs[b].level;
    flags[b] = 0;
    if (aret >= 0) a->deref[b] = 0;
    if (aret > 0) {
      flags[b] = level == a->max_level ? 0 : 1;
    } else if (aret < 0) {
      if (level == root) {
        a->deref[b] = 0;
      } else {
        a->deref[b] += 1;
        bool finer = false;
        for (int q = 0; q < 27; ++q)
          if (a->nblevel[b * 27 + q] > level) finer = true;
        if (!finer && a->deref[b] >= a->derefine_count) flags[b] = -1;
      }
    }
  }
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_update(athgpu_amr* a, const int* flags, int* changed) {
  if (!a || !flags || !changed) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *changed = 0;
  a->pending = false;
  const size_t nb = a->locs.size();
  std::vector<Loc> lref, lderef;
  for (size_t b = 0; b < nb; ++b) {
    if (flags[b] == 1) lref.push_back(a->locs[b]);
    if (flags[b] == -1) lderef.push_back(a->locs[b]);
  }
  const int nleaf = 8;
  if (lref.empty() && (int)lderef.size() < nleaf) return ATHGPU_OK;
  // groups of eight flagged siblings in gid order (amr_loadbalance.cpp:255-283)
  std::vector<Loc> clderef;
  const int tn = (int)lderef.size();
  if (tn >= nleaf)
    for (int n = 0; n < tn; ++n) {
      const Loc& L = lderef[n];
      if ((L.lx[0] & 1) || (L.lx[1] & 1) || (L.lx[2] & 1)) continue;
      int r = n, rr = 0;
      for (int k = 0; k <= 1; ++k)
        for (int j = 0; j <= 1; ++j)
          for (int i = 0; i <= 1; ++i)
            if (r < tn) {
              const Loc& R = lderef[r];
              if (L.lx[0] + i == R.lx[0] && L.lx[1] + j == R.lx[1] && L.lx[2] + k == R.lx[2] &&
                  L.level == R.level)
                ++rr;
              ++r;
            }
      if (rr == nleaf)
        clderef.push_back(Loc{L.level - 1, {L.lx[0] >> 1, L.lx[1] >> 1, L.lx[2] >> 1}});
    }
  // by decreasing level over all but the last group (the reference's sort range,
  // amr_loadbalance.cpp:286-287); equal levels keep their order
  if (clderef.size() > 1)
    std::stable_sort(clderef.begin(), clderef.end() - 1,
                     [](const Loc& x, const Loc& y) { return x.level > y.level; });
  BlockTree& t = a->tree;
  t.nnew = t.ndel = 0;
  for (const Loc& L : lref) {
    const int nd = t.find(L);
    if (nd >= 0) t.refine(nd);
  }
  for (const Loc& L : clderef) {
    const int nd = t.find(L);
    if (nd >= 0 && t.nodes[nd].refined && t.derefine_ok(nd)) t.derefine(nd);
  }
  if (t.nnew == 0 && t.ndel == 0) return ATHGPU_OK;
  std::vector<int> old;
  t.block_list(&a->new_locs, &old);
  const size_t nn = a->new_locs.size();
  a->newtoold.assign(old.begin(), old.end());
  a->kind.assign(nn, 0);
  a->new_deref.assign(nn, 0);
  for (size_t n = 0; n < nn; ++n) {
    const int on = old[n];
    if (on < 0 || on >= (int)nb) return api_fail(ATHGPU_ERR_ARG, "tree update lost a block");
    const int ol = a->locs[on].level, nl = a->new_locs[n].level;
    if (nl == ol) {
      a->new_deref[n] = a->deref[on];
    } else {
      a->kind[n] = nl < ol ? 1 : 2;
    }
  }
  // face-field corrections (amr_loadbalance.cpp:1225-1340)
  std::map<Loc, int> oldmap;
  for (size_t i = 0; i < nb; ++i)
    if (a->locs[i].level > t.root_level) oldmap[a->locs[i]] = (int)i;
  a->ffc.clear();
  for (size_t n = 0; n < nn; ++n) {
    if (a->kind[n] != 2) continue;
    const Loc& nl = a->new_locs[n];
    for (int d = 0; d < 3; ++d) {
      const int xf = (int)(nl.lx[d] & 1);
      Loc f = nl;
      f.lx[d] += 2 * xf - 1;
      const long long nmax = t.nblocks_at(d, nl.level);
      if (f.lx[d] < 0) {
        if (a->g.bcs[2 * d] != 0) continue;
        f.lx[d] = nmax - 1;
      } else if (f.lx[d] >= nmax) {
        if (a->g.bcs[2 * d + 1] != 0) continue;
        f.lx[d] = 0;
      }
      auto it = oldmap.find(f);
      if (it != oldmap.end()) {
        a->ffc.push_back((int)n);
        a->ffc.push_back(2 * d + xf);
        a->ffc.push_back(it->second);
      }
    }
  }
  a->pending = true;
  *changed = 1;
  return ATHGPU_OK;
}

// the pending plan's maps (sizes from athgpu_amr_pending)
athgpu_status athgpu_amr_pending(const athgpu_amr* a, int* nblocks_new, int* nffc) {
  if (!a || !nblocks_new || !nffc) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *nblocks_new = a->pending ? (int)a->new_locs.size() : 0;
  *nffc = a->pending ? (int)a->ffc.size() / 3 : 0;
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_pending_maps(const athgpu_amr* a, int* newtoold, int* kind, int* ffc,
                                      int* deref_count) {
  if (!a || !a->pending) return api_fail(ATHGPU_ERR_STATE, "no pending regrid");
  if (newtoold) std::memcpy(newtoold, a->newtoold.data(), sizeof(int) * a->newtoold.size());
  if (kind) std::memcpy(kind, a->kind.data(), sizeof(int) * a->kind.size());
  if (ffc) std::memcpy(ffc, a->ffc.data(), sizeof(int) * a->ffc.size());
  if (deref_count) std::memcpy(deref_count, a->new_deref.data(), sizeof(int) * a->new_deref.size());
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_accept(athgpu_amr* a) {
  if (!a || !a->pending) return api_fail(ATHGPU_ERR_STATE, "no pending regrid");
  a->locs.swap(a->new_locs);
  a->deref.swap(a->new_deref);
  a->pending = false;
  if (!a->rebuild_tables(a->locs, &a->table, &a->count, &a->nblevel))
    return api_fail(ATHGPU_ERR_ARG, "neighbour search failed");
  return ATHGPU_OK;
}

athgpu_status athgpu_amr_deref_counts(const athgpu_amr* a, int* out) {
  if (!a || !out) return api_fail(ATHGPU_ERR_ARG, "null argument");
  std::memcpy(out, a->deref.data(), sizeof(int) * a->deref.size());
  return ATHGPU_OK;
}

namespace athgpu {
athgpu_status ctx_desc(athgpu_ctx* c, athgpu_mesh_desc* out);
}

// One refinement check and regrid (the end of a main-loop cycle: the last stage's
// CheckRefinementCondition, LoadBalancingAndAdaptiveMeshRefinement and, with
// after_cycle, the main loop's NewTimeStep) with the blast problem's condition
// (pgen/blast.cpp:413-443) at threshold thr.
athgpu_status athgpu_amr_step(athgpu_ctx* ctx, athgpu_amr* a, double thr, int after_cycle,
                              int* regridded) {
  if (!ctx || !a || !regridded) return api_fail(ATHGPU_ERR_ARG, "null argument");
  *regridded = 0;
  const size_t nb = a->locs.size();
  athgpu_mesh_desc d;
  athgpu_status st = athgpu::ctx_desc(ctx, &d);
  if (st != ATHGPU_OK) return st;
  if ((size_t)d.nbx1 != nb) return api_fail(ATHGPU_ERR_ARG, "context and adaptive mesh differ");
  std::vector<double> eps(nb);
  st = athgpu_refinement_eps(ctx, eps.data());
  if (st != ATHGPU_OK) return st;
  std::vector<int> ret(nb), flags(nb);
  for (size_t b = 0; b < nb; ++b)
    ret[b] = eps[b] > thr ? 1 : (eps[b] < 0.25 * thr ? -1 : 0);
  athgpu_amr_flags(a, ret.data(), flags.data());
  int changed = 0;
  st = athgpu_amr_update(a, flags.data(), &changed);
  if (st != ATHGPU_OK || !changed) return st;
  std::vector<int> newtoold(a->newtoold), kind(a->kind), ffc(a->ffc);
  st = athgpu_amr_accept(a);
  if (st != ATHGPU_OK) return st;
  const size_t nn = a->locs.size();
  std::vector<long long> loc(nn * 4);
  std::vector<int> table(a->table), count(a->count), nblevel(a->nblevel);
  std::vector<double> f[6], cf[6];
  for (int q = 0; q < 3; ++q) {
    const int nc = a->g.bx[q] + 2 * a->g.ng, ncc = a->g.bx[q] / 2 + 2 * a->g.ng;
    f[2 * q].resize(nn * (nc + 1));
    f[2 * q + 1].resize(nn * nc);
    cf[2 * q].resize(nn * (ncc + 1));
    cf[2 * q + 1].resize(nn * ncc);
  }
  double* const fp[6] = {f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data(), f[5].data()};
  double* const cp[6] = {cf[0].data(), cf[1].data(), cf[2].data(), cf[3].data(), cf[4].data(),
                         cf[5].data()};
  fill_tables(a, loc.data(), nullptr, nullptr, nullptr, fp, cp);
  d.nbx1 = (int)nn;
  d.nbx2 = d.nbx3 = 1;
  d.x1f = fp[0]; d.dx1f = fp[1]; d.x2f = fp[2]; d.dx2f = fp[3]; d.x3f = fp[4]; d.dx3f = fp[5];
  st = athgpu_regrid(ctx, &d, table.data(), count.data(), nblevel.data(), loc.data(), cp[0],
                     cp[1], cp[2], cp[3], cp[4], cp[5], newtoold.data(), kind.data(),
                     (int)(ffc.size() / 3), ffc.data(), after_cycle);
  if (st != ATHGPU_OK) return st;
  if (after_cycle) {
    st = athgpu_new_time_step(ctx);
    if (st != ATHGPU_OK) return st;
  }
  *regridded = 1;
  return ATHGPU_OK;
}
