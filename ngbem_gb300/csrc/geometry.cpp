// Mesh, trace spaces, cluster trees and the block partition.
//
// The cluster tree restates the reference's Rjasanow PCA bisection bit for bit
// (ComputeClusterData src/hmat.cpp:13-150, Rja_DivideCluster :155-374, Rja_ClusterTree
// :379-407, ClusterTree ctor :409-453) with a documented 3x3 eigen solver in place of LAPACK
// dsyev; the partition restates Rja_AdmissiblePair (:457-471) and HMatrix_help (:587-612).
#include <algorithm>
#include <thread>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <exception>
#include <functional>
#include <numeric>
#include <unordered_map>

#include "host.hpp"

namespace bem {

// ------------------------------------------------------------------------------------------
// mesh
// ------------------------------------------------------------------------------------------
void MeshH::build(int nv_, const double* xyz, int nt_, const int* tri) {
  if (nv_ <= 0 || nt_ <= 0) throw Error(BEM_ERR_ARG, "mesh needs vertices and triangles");
  nv = nv_;
  nt = nt_;
  X.assign(xyz, xyz + 3 * (size_t)nv);
  T.assign(tri, tri + 3 * (size_t)nt);
  for (int k = 0; k < 3 * nt; ++k)
    if (T[k] < 0 || T[k] >= nv) throw Error(BEM_ERR_ARG, "triangle vertex index out of range");
  // edges by first appearance: elements in order, local edges (0,1),(1,2),(2,0)
  std::unordered_map<long long, int> ids;
  ids.reserve((size_t)nt * 2);
  TE.resize(3 * (size_t)nt);
  E.clear();
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < 3; ++k) {
      int a = T[3 * e + k], b = T[3 * e + (k + 1) % 3];
      int lo = std::min(a, b), hi = std::max(a, b);
      long long key = (long long)lo * nv + hi;
      auto it = ids.find(key);
      int id;
      if (it == ids.end()) {
        id = (int)(E.size() / 2);
        ids.emplace(key, id);
        E.push_back(lo);
        E.push_back(hi);
      } else {
        id = it->second;
      }
      TE[3 * e + k] = id;
    }
  ne = (int)(E.size() / 2);
  rec.resize(nt);
  for (int e = 0; e < nt; ++e) {
    ElemRec64& r = rec[e];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) r.p[k][c] = X[3 * (size_t)T[3 * e + k] + c];
    double J0[3], J1[3];
    for (int c = 0; c < 3; ++c) {
      J0[c] = r.p[0][c] - r.p[2][c];
      J1[c] = r.p[1][c] - r.p[2][c];
    }
    const double cr[3] = {J0[1] * J1[2] - J0[2] * J1[1], J0[2] * J1[0] - J0[0] * J1[2], J0[0] * J1[1] - J0[1] * J1[0]};
    r.detJ = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    if (!(r.detJ > 0.0)) throw Error(BEM_ERR_ARG, "degenerate triangle " + std::to_string(e));
    r.invdetJ = 1.0 / r.detJ;
    for (int c = 0; c < 3; ++c) r.n[c] = cr[c] / r.detJ;
    // surface gradients of the hat functions: J (J^T J)^{-1} grad_ref, rotated by n x .
    const double g00 = J0[0] * J0[0] + J0[1] * J0[1] + J0[2] * J0[2];
    const double g01 = J0[0] * J1[0] + J0[1] * J1[1] + J0[2] * J1[2];
    const double g11 = J1[0] * J1[0] + J1[1] * J1[1] + J1[2] * J1[2];
    const double det = g00 * g11 - g01 * g01;
    const double gh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {-1.0, -1.0}};
    for (int a = 0; a < 3; ++a) {
      const double c0 = (g11 * gh[a][0] - g01 * gh[a][1]) / det;
      const double c1 = (-g01 * gh[a][0] + g00 * gh[a][1]) / det;
      double g[3];
      for (int c = 0; c < 3; ++c) g[c] = J0[c] * c0 + J1[c] * c1;
      r.rot[a][0] = r.n[1] * g[2] - r.n[2] * g[1];
      r.rot[a][1] = r.n[2] * g[0] - r.n[0] * g[2];
      r.rot[a][2] = r.n[0] * g[1] - r.n[1] * g[0];
    }
    r.pad[0] = 0.0;
  }
}

void MeshH::set_geometry(int order, const double* nodes) {
  std::lock_guard<std::mutex> lk(mu);
  if (order < 1 || order > 4) throw Error(BEM_ERR_ARG, "geometry order must be 1 to 4");
  if (order > 1 && !nodes) throw Error(BEM_ERR_ARG, "curved geometry needs its nodes");
  if (dev_ready || !tables.empty() || nspaces.load() > 0)
    throw Error(BEM_ERR_STATE, "the mesh is in use: curve it before creating spaces on it");
  gorder = order;
  G.clear();
  if (order == 1) return;
  const size_t n = (size_t)nt * 3 * gnodes();
  G.assign(nodes, nodes + n);
  for (size_t k = 0; k < n; ++k)
    if (!std::isfinite(G[k])) throw Error(BEM_ERR_ARG, "curved geometry nodes must be finite");
  // the vertices of each element are its corner nodes
  const int g = gorder, nn = gnodes();
  const int corner[3] = {0, nn - (g + 1), nn - 1};  // (g,0,0), (0,g,0), (0,0,g) in node order
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c)
        if (G[((size_t)e * nn + corner[k]) * 3 + c] != X[3 * (size_t)T[3 * e + k] + c]) {
          gorder = 1;
          G.clear();
          throw Error(BEM_ERR_ARG, "curved element " + std::to_string(e) + ": corner node differs from its vertex");
        }
  for (int e = 0; e < nt; ++e) {
    double x[3], n[3], rt[3][3];
    for (int q = 0; q < 3; ++q) {
      const double xi = q == 0 ? 1. / 3 : (q == 1 ? 0.1 : 0.8), eta = q == 0 ? 1. / 3 : 0.1;
      if (!(frame(e, xi, eta, x, n, rt) > 0.0)) {
        gorder = 1;
        G.clear();
        throw Error(BEM_ERR_ARG, "degenerate curved element " + std::to_string(e));
      }
    }
  }
}

void MeshH::map(int e, double xi, double eta, double* x) const {
  if (gorder > 1) {
    double J0[3], J1[3];
    curved_map(gorder, &G[(size_t)e * gnodes() * 3], xi, eta, x, J0, J1);
    return;
  }
  const ElemRec64& r = rec[e];
  const double l2 = 1.0 - xi - eta;
  for (int c = 0; c < 3; ++c) x[c] = xi * r.p[0][c] + eta * r.p[1][c] + l2 * r.p[2][c];
}

double MeshH::frame(int e, double xi, double eta, double* x, double* n, double rot[3][3], double* J0o,
                    double* J1o) const {
  if (gorder > 1) {
    double J0[3], J1[3];
    curved_map(gorder, &G[(size_t)e * gnodes() * 3], xi, eta, x, J0, J1);
    if (J0o)
      for (int c = 0; c < 3; ++c) { J0o[c] = J0[c]; J1o[c] = J1[c]; }
    return surface_frame(J0, J1, n, rot);
  }
  const ElemRec64& r = rec[e];
  map(e, xi, eta, x);
  if (J0o)
    for (int c = 0; c < 3; ++c) { J0o[c] = r.p[0][c] - r.p[2][c]; J1o[c] = r.p[1][c] - r.p[2][c]; }
  for (int c = 0; c < 3; ++c) n[c] = r.n[c];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) rot[a][c] = r.rot[a][c];
  return r.detJ;
}

double MeshH::area(int e) const {
  if (gorder == 1) return 0.5 * rec[e].detJ;
  double x[3], n[3], rt[3][3];
  return 0.5 * frame(e, 1. / 3, 1. / 3, x, n, rt);
}

void MeshH::ensure_device() {
  std::lock_guard<std::mutex> lk(mu);
  if (dev_ready) return;
  std::vector<int4> t4(nt);
  for (int e = 0; e < nt; ++e) t4[e] = make_int4(T[3 * e], T[3 * e + 1], T[3 * e + 2], 0);
  d_tri.upload(t4);
  d_rec64.upload(rec);
  if (gorder > 1) d_gnodes.upload(G);
  BEM_CUDA(cudaDeviceSynchronize());
  dev_ready = true;
}

template <class P>
static void build_tables(const MeshH& m, const TrigRule& r, std::vector<ElemRecP<P>>& recs,
                         std::vector<QPt<P>>& qoff, std::vector<APt<P>>& apts, std::vector<P>& rq,
                         std::vector<PGeo<P>>& pgeo) {
  const int nq = (int)r.w.size();
  recs.resize(m.nt);
  qoff.resize((size_t)m.nt * nq);
  apts.resize((size_t)m.nt * nq);
  pgeo.resize(m.curved() ? (size_t)m.nt * nq : 0);
  rq.resize(2 * nq);
  for (int q = 0; q < nq; ++q) {
    rq[2 * q] = (P)r.xi[q];
    rq[2 * q + 1] = (P)r.eta[q];
  }
  for (int e = 0; e < m.nt; ++e) {
    const ElemRec64& s = m.rec[e];
    ElemRecP<P>& d = recs[e];
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = (s.p[0][k] + s.p[1][k] + s.p[2][k]) / 3.0;
    for (int k = 0; k < 3; ++k) {
      d.chi[k] = (P)c[k];
      d.clo[k] = (P)(c[k] - (double)d.chi[k]);
      d.n[k] = (P)s.n[k];
    }
    d.detJ = (P)s.detJ;
    d.invdetJ = (P)s.invdetJ;
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) {
        d.o[a][k] = (P)(s.p[a][k] - c[k]);
        d.rot[a][k] = (P)s.rot[a][k];
      }
    d.pad[0] = d.pad[1] = d.pad[2] = (P)0;
    for (int q = 0; q < nq; ++q) {
      // the point, and w |J| at it (curved elements: their normal and rotated gradients too)
      double x[3], nq3[3], rt[3][3], J0[3], J1[3];
      const double detJ = m.frame(e, r.xi[q], r.eta[q], x, nq3, rt, J0, J1);
      const double w = r.w[q] * detJ;
      if (m.curved()) {
        PGeo<P>& g = pgeo[(size_t)e * nq + q];
        double xp[3][3];
        piola_offsets(J0, J1, r.xi[q], r.eta[q], xp);
        g.invdetJ = (P)(1.0 / detJ);
        for (int c = 0; c < 3; ++c) {
          g.n[c] = (P)nq3[c];
          for (int a = 0; a < 3; ++a) {
            g.rot[a][c] = (P)rt[a][c];
            g.xp[a][c] = (P)xp[a][c];
          }
        }
      }
      QPt<P>& qo = qoff[(size_t)e * nq + q];
      qo.x = (P)(x[0] - c[0]);
      qo.y = (P)(x[1] - c[1]);
      qo.z = (P)(x[2] - c[2]);
      qo.w = (P)w;
      APt<P>& ap = apts[(size_t)e * nq + q];
      ap.hx = (P)x[0];
      ap.hy = (P)x[1];
      ap.hz = (P)x[2];
      ap.lx = (P)(x[0] - (double)ap.hx);
      ap.ly = (P)(x[1] - (double)ap.hy);
      ap.lz = (P)(x[2] - (double)ap.hz);
      ap.w = (P)w;
      ap.pad = (P)0;
    }
  }
}

MeshH::RuleTables& MeshH::rule_tables(int order) {
  ensure_device();
  std::lock_guard<std::mutex> lk(mu);
  auto it = tables.find(order);
  if (it != tables.end()) return *it->second;
  auto t = std::make_unique<RuleTables>();
  TrigRule r = make_trig_rule(order);
  t->nq = (int)r.w.size();
  {
    std::vector<ElemRecP<double>> recs;
    std::vector<QPt<double>> qo;
    std::vector<APt<double>> ap;
    std::vector<double> rq;
    std::vector<PGeo<double>> pg;
    build_tables<double>(*this, r, recs, qo, ap, rq, pg);
    if (!pg.empty()) t->pgeo[0].upload(pg);
    t->rec[0].upload(recs);
    t->qoff[0].upload(qo);
    t->apts[0].upload(ap);
    t->rq[0].upload(rq);
    BEM_CUDA(cudaDeviceSynchronize());
  }
  {
    std::vector<ElemRecP<float>> recs;
    std::vector<QPt<float>> qo;
    std::vector<APt<float>> ap;
    std::vector<float> rq;
    std::vector<PGeo<float>> pg;
    build_tables<float>(*this, r, recs, qo, ap, rq, pg);
    if (!pg.empty()) t->pgeo[1].upload(pg);
    t->rec[1].upload(recs);
    t->qoff[1].upload(qo);
    t->apts[1].upload(ap);
    t->rq[1].upload(rq);
    BEM_CUDA(cudaDeviceSynchronize());
  }
  auto& ref = *t;
  tables[order] = std::move(t);
  return ref;
}

// ------------------------------------------------------------------------------------------
// trace spaces
// ------------------------------------------------------------------------------------------
void SpaceH::build(MeshH* m, int kind_, int dual_, const unsigned char* mask) {
  mesh = m;
  m->nspaces.fetch_add(1);
  kind = kind_;
  dual = dual_ ? 1 : 0;
  elems.clear();
  for (int e = 0; e < m->nt; ++e)
    if (!mask || mask[e]) elems.push_back(e);
  if (elems.empty()) throw Error(BEM_ERR_ARG, "the space's region has no elements");
  dofs.assign(3 * (size_t)m->nt, -1);
  sign.assign(3 * (size_t)m->nt, 1);
  global_dof.clear();
  // On a region the dofs are numbered like those of the mesh made of the region's elements
  // (in element order, vertices renumbered in ascending order): P0 the elements in order, P1
  // the vertices in ascending order, RT0 / HCURL the edges by first appearance.
  if (kind == BEM_P0) {
    nd = 1;
    for (int e : elems) {
      dofs[3 * e] = dofs[3 * e + 1] = dofs[3 * e + 2] = (int)global_dof.size();
      global_dof.push_back(e);
    }
  } else if (kind == BEM_P1) {
    nd = 3;
    std::vector<int> map(m->nv, -1);
    for (int e : elems)
      for (int k = 0; k < 3; ++k) map[m->T[3 * e + k]] = 0;
    for (int v = 0; v < m->nv; ++v)
      if (map[v] == 0) {
        map[v] = (int)global_dof.size();
        global_dof.push_back(v);
      }
    for (int e : elems)
      for (int k = 0; k < 3; ++k) dofs[3 * e + k] = map[m->T[3 * e + k]];
  } else if (kind == BEM_RT0 || kind == BEM_HCURL) {
    nd = 3;
    std::vector<int> map(m->ne, -1);
    for (int e : elems)
      for (int k = 0; k < 3; ++k) {
        const int g = m->TE[3 * e + k];
        if (map[g] < 0) {
          map[g] = (int)global_dof.size();
          global_dof.push_back(g);
        }
        dofs[3 * e + k] = map[g];
        sign[3 * e + k] = m->T[3 * e + k] < m->T[3 * e + (k + 1) % 3] ? 1 : -1;
      }
  } else if (kind >= BEM_L2P1 && kind <= BEM_L2P3) {
    // SurfaceL2 of order p: (p+1)(p+2)/2 consecutive dofs per element; the signs hold the
    // element's local vertices in the order of their global numbers (the Dubiner basis is
    // built on that order, as NGSolve's L2 triangle element builds it)
    const int p = kind - BEM_L2P1 + 1;
    nd = (p + 1) * (p + 2) / 2;
    for (int e : elems) {
      dofs[3 * e] = dofs[3 * e + 1] = dofs[3 * e + 2] = (int)global_dof.size();
      for (int a = 0; a < nd; ++a) global_dof.push_back(e);
      int f[3] = {0, 1, 2};
      std::sort(f, f + 3, [&](int x, int y) { return m->T[3 * e + x] < m->T[3 * e + y]; });
      for (int k = 0; k < 3; ++k) sign[3 * e + k] = f[k];
    }
  } else if (kind == BEM_H1P2 || kind == BEM_H1P3) {
    // H1 of order p: vertex dofs (vertices ascending), p - 1 per edge (edges by first
    // appearance on the region), (p - 1)(p - 2) / 2 per element; sign: the orientation of
    // local edge k (+1 when its first vertex has the lower global number).  global_dof: the
    // dof of the same function in the space on the whole mesh (edges in mesh order).
    const int p = kind == BEM_H1P2 ? 2 : 3, pe = p - 1, pf = (p - 1) * (p - 2) / 2;
    nd = (p + 1) * (p + 2) / 2;
    xdof.assign((size_t)nd * m->nt, -1);
    std::vector<int> vmap(m->nv, -1), emap(m->ne, -1);
    for (int e : elems)
      for (int k = 0; k < 3; ++k) vmap[m->T[3 * e + k]] = 0;
    for (int v = 0; v < m->nv; ++v)
      if (vmap[v] == 0) {
        vmap[v] = (int)global_dof.size();
        global_dof.push_back(v);
      }
    for (int e : elems)
      for (int k = 0; k < 3; ++k) {
        const int g = m->TE[3 * e + k];
        if (emap[g] < 0) {
          emap[g] = (int)global_dof.size();
          for (int j = 0; j < pe; ++j) global_dof.push_back(m->nv + g * pe + j);
        }
      }
    for (int e : elems) {
      const int f0 = (int)global_dof.size();
      for (int j = 0; j < pf; ++j) global_dof.push_back(m->nv + m->ne * pe + e * pf + j);
      int* xd = &xdof[(size_t)nd * e];
      for (int k = 0; k < 3; ++k) {
        dofs[3 * e + k] = vmap[m->T[3 * e + k]];
        sign[3 * e + k] = m->T[3 * e + k] < m->T[3 * e + (k + 1) % 3] ? 1 : -1;
        xd[k] = dofs[3 * e + k];
        for (int j = 0; j < pe; ++j) xd[3 + k * pe + j] = emap[m->TE[3 * e + k]] + j;
      }
      for (int j = 0; j < pf; ++j) xd[3 + 3 * pe + j] = f0 + j;
    }
  } else if (bdm_kind_order(kind) > 0) {
    // HDivSurface of order K: the lowest-order dofs of the edges (by first appearance on the
    // region), then K per edge in the same order, then (K + 1)(K - 1) per element; local dofs
    // per edge k (K + 1 of them), then the interior ones (hdiv_shape); sign: the orientation of
    // local edge k.  global_dof: the dof of the same function in the space on the whole mesh.
    const int K = bdm_kind_order(kind), nin = (K + 1) * (K - 1);
    nd = (K + 1) * (K + 2);
    xdof.assign((size_t)nd * m->nt, -1);
    std::vector<int> emap(m->ne, -1), eord;
    for (int e : elems)
      for (int k = 0; k < 3; ++k) {
        const int g = m->TE[3 * e + k];
        if (emap[g] < 0) {
          emap[g] = (int)eord.size();
          eord.push_back(g);
        }
      }
    const int nlo = (int)eord.size();
    for (int g : eord) global_dof.push_back(g);
    for (int g : eord)
      for (int j = 0; j < K; ++j) global_dof.push_back(m->ne + g * K + j);
    for (int e : elems)
      for (int j = 0; j < nin; ++j) global_dof.push_back(m->ne * (K + 1) + e * nin + j);
    int ei = 0;
    for (int e : elems) {
      int* xd = &xdof[(size_t)nd * e];
      for (int k = 0; k < 3; ++k) {
        const int lo = emap[m->TE[3 * e + k]];
        dofs[3 * e + k] = lo;
        sign[3 * e + k] = m->T[3 * e + k] < m->T[3 * e + (k + 1) % 3] ? 1 : -1;
        xd[k * (K + 1)] = lo;
        for (int j = 0; j < K; ++j) xd[k * (K + 1) + 1 + j] = nlo + lo * K + j;
      }
      for (int j = 0; j < nin; ++j) xd[3 * (K + 1) + j] = nlo * (K + 1) + ei * nin + j;
      ++ei;
    }
  } else {
    throw Error(BEM_ERR_ARG, "unknown space kind");
  }
  ndof = (int)global_dof.size();
  // dof -> elements (CSR, ascending element ids)
  e4d_ptr.assign(ndof + 1, 0);
  for (int e : elems)
    for (int a = 0; a < nd; ++a) e4d_ptr[dof(e, a) + 1]++;
  for (int d = 0; d < ndof; ++d) e4d_ptr[d + 1] += e4d_ptr[d];
  e4d.assign(e4d_ptr[ndof], 0);
  std::vector<int> fill(e4d_ptr.begin(), e4d_ptr.end() - 1);
  for (int e : elems)
    for (int a = 0; a < nd; ++a) e4d[fill[dof(e, a)]++] = e;
  for (int d = 0; d < ndof; ++d)
    if (e4d_ptr[d + 1] == e4d_ptr[d]) throw Error(BEM_ERR_ARG, "space has a dof without elements");
}

void SpaceH::ensure_device() {
  if (d_dofs.p) return;
  std::vector<int4> d4(mesh->nt), s4(mesh->nt);
  for (int e = 0; e < mesh->nt; ++e) {
    d4[e] = make_int4(dofs[3 * e], dofs[3 * e + 1], dofs[3 * e + 2], 0);
    s4[e] = make_int4(sign[3 * e], sign[3 * e + 1], sign[3 * e + 2], 0);
    if ((kind == BEM_H1P2 || kind == BEM_H1P3) && on(e)) {
      // H1 of order p: w = the first face dof; the signs carry (first edge dof + 1)
      const int pe = nd == 6 ? 1 : 2;
      const int* xd = &xdof[(size_t)nd * e];
      d4[e].w = nd > 3 + 3 * pe ? xd[3 + 3 * pe] : 0;
      s4[e] = make_int4(sign[3 * e] * (xd[3] + 1), sign[3 * e + 1] * (xd[3 + pe] + 1),
                        sign[3 * e + 2] * (xd[3 + 2 * pe] + 1), 0);
    }
    if (bdm_kind_order(kind) > 0 && on(e)) {
      // HDivSurface and HCurl of order K: w = the first interior dof; the signs carry (first
      // higher-order dof of the edge + 1)
      const int K = bdm_kind_order(kind);
      const int* xd = &xdof[(size_t)nd * e];
      d4[e].w = nd > 3 * (K + 1) ? xd[3 * (K + 1)] : 0;
      s4[e] = make_int4(sign[3 * e] * (xd[1] + 1), sign[3 * e + 1] * (xd[K + 2] + 1),
                        sign[3 * e + 2] * (xd[2 * K + 3] + 1), 0);
    }
  }
  d_dofs.upload(d4);
  d_sign.upload(s4);
  BEM_CUDA(cudaDeviceSynchronize());
}

int trace_kind(int space_kind, int ev) {
  if (space_kind == BEM_P0) return ev == BEM_EV_ID ? TR_P0 : -1;
  if (space_kind >= BEM_L2P1 && space_kind <= BEM_L2P3) return ev == BEM_EV_ID ? TR_L2P1 + space_kind - BEM_L2P1 : -1;
  if (space_kind == BEM_H1P2 || space_kind == BEM_H1P3) {
    const int q = space_kind - BEM_H1P2;
    if (ev == BEM_EV_ID) return TR_H1P2 + q;
    if (ev == BEM_EV_ROT) return TR_H1P2ROT + q;
    if (ev == BEM_EV_HELM) return TR_H1P2HELM + q;
    return -1;
  }
  if (space_kind == BEM_P1) {
    if (ev == BEM_EV_ID) return TR_P1;
    if (ev == BEM_EV_ROT) return TR_ROT;
    if (ev == BEM_EV_HELM) return TR_HELM;
    return -1;
  }
  if (space_kind == BEM_RT0) {
    if (ev == BEM_EV_MAXWELL) return TR_MAX;
    if (ev == BEM_EV_ID) return TR_RT0ID;
    return -1;
  }
  if (const int K = bdm_kind_order(space_kind)) {
    if (!bdm_kind_curl(space_kind)) {
      if (ev == BEM_EV_ID) return bdm_trace(K, false, 0);
      if (ev == BEM_EV_MAXWELL) return bdm_trace(K, false, 1);
      return -1;
    }
    if (ev == BEM_EV_ID) return bdm_trace(K, true, 0);
    if (ev == BEM_EV_ROTATED_TRACE) return bdm_trace(K, true, 1);
    if (ev == BEM_EV_MAXWELL_CURL) return bdm_trace(K, true, 2);
    return -1;
  }
  if (space_kind == BEM_HCURL) {
    if (ev == BEM_EV_ID) return TR_NED;
    if (ev == BEM_EV_ROTATED_TRACE) return TR_NEDROT;
    if (ev == BEM_EV_MAXWELL_CURL) return TR_NEDMAX;
    return -1;
  }
  return -1;
}

// ------------------------------------------------------------------------------------------
// cluster tree
// ------------------------------------------------------------------------------------------
// ComputeClusterData: dof weights (mean adjacent area) and points (vertex if the dof has more
// than two elements, edge midpoint if two, centroid if one); the last element wins.
static void cluster_data(const SpaceH& sp, std::vector<double>& G, std::vector<std::array<double, 3>>& X) {
  const MeshH& m = *sp.mesh;
  const int ndof = sp.ndof;
  G.assign(ndof, 0.0);
  X.assign(ndof, {0.0, 0.0, 0.0});
  std::vector<int> cnt(ndof, 0);
  for (int e : sp.elems)
    for (int a = 0; a < sp.nd; ++a) {
      const int d = sp.dof(e, a);
      G[d] += m.area(e);
      cnt[d] += 1;
    }
  static const double xhat[7][2] = {{1, 0}, {0, 1}, {0, 0}, {0.5, 0.5}, {0, 0.5}, {0.5, 0}, {1. / 3, 1. / 3}};
  for (int e : sp.elems) {
    double pt[7][3];
    for (int j = 0; j < 7; ++j) m.map(e, xhat[j][0], xhat[j][1], pt[j]);
    auto dn = [&](int a) { return sp.dof(e, a); };
    int nvert = 0, nedge = 0;
    for (int a = 0; a < sp.nd; ++a) {
      const int c = cnt[dn(a)];
      if (c > 2) { X[dn(a)] = {pt[nvert][0], pt[nvert][1], pt[nvert][2]}; ++nvert; }
      if (c == 2) ++nedge;
      if (c == 1) X[dn(a)] = {pt[6][0], pt[6][1], pt[6][2]};
    }
    // fewer than three two-element dofs (an element at the border of an open surface or of a
    // region): each is its own edge (the reference's loop would not advance with 0 per edge)
    const int per_edge = std::max(1, nedge / 3);
    int ie = 0;
    for (int a = 0; a < sp.nd; ++a) {
      if (cnt[dn(a)] != 2) continue;
      for (int o = 0; o < per_edge; ++o) X[dn(a + o)] = {pt[3 + ie][0], pt[3 + ie][1], pt[3 + ie][2]};
      ++ie;
      a += per_edge - 1;
    }
  }
  for (int i = 0; i < ndof; ++i) G[i] /= (double)cnt[i];
}

// cluster trees of at least this many dofs are built on a team of host threads
static const int kTreeTeamMinDofs = 4096;

// Host threads kept for the levels of one tree build (starting threads per level cost more
// than a level's work at 20k dofs).  run(n, f) calls f(i) for i in [0, n) on the team and
// the calling thread and returns when every call has returned; an exception from f is
// rethrown there after the team has stopped touching f.
class LevelTeam {
 public:
  explicit LevelTeam(int workers) {
    for (int t = 0; t < workers; ++t) {
      try {
        th_.emplace_back([this] { loop(); });
      } catch (...) {
        break;  // no more threads to be had: the team works with those it has (or none)
      }
    }
  }
  ~LevelTeam() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(int n, const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      n_ = n;
      next_.store(0);
      busy_ = (int)th_.size();
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [this] { return busy_ == 0; });
    job_ = nullptr;
    if (failure_) {
      std::exception_ptr e = failure_;
      failure_ = nullptr;
      std::rethrow_exception(e);
    }
  }

 private:
  void work() {
    try {
      for (int i = next_++; i < n_; i = next_++) (*job_)(i);
    } catch (...) {
      next_.store(n_);  // the others stop taking items
      std::lock_guard<std::mutex> lk(mu_);
      if (!failure_) failure_ = std::current_exception();
    }
  }
  void loop() {
    long long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
      }
      work();
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_.notify_one();
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0, busy_ = 0;
  long long gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
  std::exception_ptr failure_;
};

// a team for a tree of n dofs (null below kTreeTeamMinDofs or on one core)
static std::unique_ptr<LevelTeam> make_tree_team(int n) {
  const int hw = (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
  if (n < kTreeTeamMinDofs || hw < 2) return nullptr;
  return std::make_unique<LevelTeam>(hw - 1);
}

// PCA bisection tree (reference Rja_ClusterTree, src/hmat.cpp:155-407), breadth first.  The
// clusters of one level own disjoint ranges of the permutation, so a level is split on parallel
// threads; the children are then appended in cluster order, which gives the numbering of the
// one-cluster-at-a-time traversal.  Each cluster's arithmetic is the serial one (bit-identical).
void ClusterTreeH::build(const SpaceH& sp, int leafsize, LevelTeam* team) {
  std::vector<double> G;
  std::vector<std::array<double, 3>> X;
  cluster_data(sp, G, X);
  const int n = sp.ndof;
  perm.resize(n);
  std::iota(perm.begin(), perm.end(), 0);
  cl.clear();
  ClusterH root;
  root.Number = n;
  cl.push_back(root);
  struct Split { int n1 = 0, n2 = 0; bool split = false; };
  auto process = [&](size_t ic, Split& out) {
    const int cnum = (int)cl[ic].Number;
    const int b = (int)cl[ic].PermuPos;
    const int e = b + cnum - 1;
    double mom[10] = {0.};
    for (int i = b; i <= e; ++i) {
      const int j = perm[i];
      mom[0] += G[j];
      mom[1] += G[j] * X[j][0];
      mom[2] += G[j] * X[j][1];
      mom[3] += G[j] * X[j][2];
      mom[4] += G[j] * X[j][0] * X[j][0];
      mom[5] += G[j] * X[j][0] * X[j][1];
      mom[6] += G[j] * X[j][0] * X[j][2];
      mom[7] += G[j] * X[j][1] * X[j][1];
      mom[8] += G[j] * X[j][1] * X[j][2];
      mom[9] += G[j] * X[j][2] * X[j][2];
    }
    const double ctr[3] = {mom[1] / mom[0], mom[2] / mom[0], mom[3] / mom[0]};
    double cov[9];
    cov[0] = mom[4] - ctr[0] * mom[1];
    cov[1] = mom[5] - ctr[0] * mom[2];
    cov[2] = mom[6] - ctr[0] * mom[3];
    cov[3] = cov[1];
    cov[4] = mom[7] - ctr[1] * mom[2];
    cov[5] = mom[8] - ctr[1] * mom[3];
    cov[6] = cov[2];
    cov[7] = cov[5];
    cov[8] = mom[9] - ctr[2] * mom[3];
    double W[3], A[9];
    sym_eigen3(cov, W, A);

    int jmin = 0;
    double xmin[3] = {0, 0, 0}, xmax[3] = {0, 0, 0};
    double r2max = 0.0, dmin = 0.0;
    for (int i = b; i <= e; ++i) {
      const int j = perm[i];
      const double df[3] = {X[j][0] - ctr[0], X[j][1] - ctr[1], X[j][2] - ctr[2]};
      const double dist = std::sqrt(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
      if (i == b || dist < dmin) { jmin = j; dmin = dist; }
      double xt[3];
      for (int r = 0; r < 3; ++r) xt[r] = A[3 * r] * df[0] + A[3 * r + 1] * df[1] + A[3 * r + 2] * df[2];
      // max of the squares, one square root at the end: sqrt is monotone and correctly rounded,
      // so this is the maximum of the square roots bit for bit
      r2max = std::fmax(r2max, xt[0] * xt[0] + xt[1] * xt[1] + xt[2] * xt[2]);
      if (i == b) {
        for (int r = 0; r < 3; ++r) xmin[r] = xmax[r] = xt[r];
      } else {
        for (int r = 0; r < 3; ++r) {
          xmin[r] = std::fmin(xmin[r], xt[r]);
          xmax[r] = std::fmax(xmax[r], xt[r]);
        }
      }
    }
    const double radius = std::sqrt(r2max);
    const double dg[3] = {xmax[0] - xmin[0], xmax[1] - xmin[1], xmax[2] - xmin[2]};
    {
      ClusterH& C = cl[ic];
      C.BasisElement = jmin;
      C.Radius = radius;
      C.DiagLength = std::sqrt(dg[0] * dg[0] + dg[1] * dg[1] + dg[2] * dg[2]);
      for (int k = 0; k < 3; ++k) {
        C.EVal[k] = W[k];
        C.XMin[k] = xmin[k];
        C.XMax[k] = xmax[k];
        C.Centre[k] = ctr[k];
      }
      for (int k = 0; k < 9; ++k) C.EVec[k] = A[k];
      C.Child1 = C.Child2 = -1;
    }
    if (cnum <= leafsize) return;
    // split on the principal axis by an in-place swap partition
    int n1 = 0, n2 = 0, chk = b, end = e;
    const double crit = ctr[0] * A[6] + ctr[1] * A[7] + ctr[2] * A[8];
    for (int i = 0; i < cnum; ++i) {
      const int j = perm[chk];
      if (X[j][0] * A[6] + X[j][1] * A[7] + X[j][2] * A[8] >= crit) {
        ++n1;
        ++chk;
      } else {
        ++n2;
        perm[chk] = perm[end];
        perm[end] = j;
        --end;
      }
    }
    out.n1 = n1;
    out.n2 = n2;
    out.split = n1 > 0 && n2 > 0;
  };
  std::vector<Split> res;
  // a team of threads for trees large enough to pay for starting it; a level runs on it when
  // it has several clusters (the top levels have one, two, ... and stay on this thread)
  std::unique_ptr<LevelTeam> own;
  if (!team) {
    own = make_tree_team(n);
    team = own.get();
  }
  for (size_t lo = 0; lo < cl.size();) {
    const size_t hi = cl.size();
    res.assign(hi - lo, Split{});
    if (team && hi - lo >= 4)
      team->run((int)(hi - lo), [&](int k) { process(lo + k, res[k]); });
    else
      for (size_t k = 0; k < hi - lo; ++k) process(lo + k, res[k]);
    for (size_t ic = lo; ic < hi; ++ic) {
      const Split& sr = res[ic - lo];
      if (!sr.split) continue;
      ClusterH c1, c2;
      c1.Level = c2.Level = cl[ic].Level + 1;
      c1.Parent = c2.Parent = (long)ic;
      c1.Number = sr.n1;
      c1.PermuPos = cl[ic].PermuPos;
      c2.Number = sr.n2;
      c2.PermuPos = cl[ic].PermuPos + sr.n1;
      cl[ic].Child1 = (long)cl.size();
      cl[ic].Child2 = (long)cl.size() + 1;
      cl.push_back(c1);
      cl.push_back(c2);
    }
    lo = hi;
  }
  pinv.assign(n, 0);
  for (int k = 0; k < n; ++k) pinv[perm[k]] = k;
}

void ClusterTreeH::build_patches(const SpaceH& sp, LevelTeam* team) {
  const int nc = (int)cl.size();
  std::unique_ptr<LevelTeam> own;
  if (!team) {
    own = make_tree_team(sp.ndof);
    team = own.get();
  }
  auto run = [&](int n, const std::function<void(int)>& f) {
    if (team && n >= 4) team->run(n, f);
    else for (int i = 0; i < n; ++i) f(i);
  };
  std::vector<std::vector<int>> pl(nc);
  auto make = [&](int c) {
    const ClusterH& C = cl[c];
    std::vector<int>& out = pl[c];
    if (sp.kind == BEM_P0) {  // one element per dof, in cluster order
      out.resize(C.Number);
      for (long k = 0; k < C.Number; ++k) out[k] = sp.global_dof[perm[C.PermuPos + k]];
      return;
    }
    if (C.Child1 >= 0) {
      const auto& a = pl[C.Child1];
      const auto& b = pl[C.Child2];
      out.reserve(a.size() + b.size());
      std::set_union(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(out));
    } else {
      for (long k = C.PermuPos; k < C.PermuPos + C.Number; ++k) {
        const int d = perm[k];
        out.insert(out.end(), sp.e4d.begin() + sp.e4d_ptr[d], sp.e4d.begin() + sp.e4d_ptr[d + 1]);
      }
      std::sort(out.begin(), out.end());
      out.erase(std::unique(out.begin(), out.end()), out.end());
    }
  };
  // levels from the deepest up (children before their parents); clusters are numbered level
  // by level, so a level is a contiguous range
  std::vector<int> lstart;
  for (int c = 0; c < nc; ++c)
    if (c == 0 || cl[c].Level != cl[c - 1].Level) lstart.push_back(c);
  lstart.push_back(nc);
  for (int l = (int)lstart.size() - 2; l >= 0; --l) {
    const int c0 = lstart[l];
    run(lstart[l + 1] - c0, [&](int k) { make(c0 + k); });
  }
  patch_ptr.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) patch_ptr[c + 1] = patch_ptr[c] + (int)pl[c].size();
  patch.resize(patch_ptr[nc]);
  patch_rad.assign(nc, 0.0);
  const MeshH& m = *sp.mesh;
  run(nc, [&](int c) {
    std::copy(pl[c].begin(), pl[c].end(), patch.begin() + patch_ptr[c]);
    double r2 = 0.0;
    for (int e : pl[c])
      for (int k = 0; k < 3; ++k) {
        const double* v = &m.X[3 * (size_t)m.T[3 * e + k]];
        const double dx = v[0] - cl[c].Centre[0], dy = v[1] - cl[c].Centre[1], dz = v[2] - cl[c].Centre[2];
        r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
      }
    patch_rad[c] = std::sqrt(r2);
  });
}

// ------------------------------------------------------------------------------------------
// partition
// ------------------------------------------------------------------------------------------
static bool admissible(const ClusterH& a, const ClusterH& b, double eta) {
  const double df[3] = {a.Centre[0] - b.Centre[0], a.Centre[1] - b.Centre[1], a.Centre[2] - b.Centre[2]};
  double dist = std::sqrt(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
  dist = std::fmax(0., dist - a.Radius - b.Radius);
  return std::fmin(a.Radius, b.Radius) < eta * dist;
}

void partition_blocks(const ClusterTreeH& row, const ClusterTreeH& col, double eta, std::vector<BlockH>& out) {
  out.clear();
  // depth-first, children in the order (1,1), (1,2), (2,1), (2,2)
  std::vector<std::pair<long, long>> stack;
  stack.push_back({0, 0});
  while (!stack.empty()) {
    auto [i, j] = stack.back();
    stack.pop_back();
    const ClusterH& rc = row.cl[i];
    const ClusterH& cc = col.cl[j];
    if (rc.Child1 == -1 || cc.Child1 == -1) {
      out.push_back({(int)i, (int)j, true});
    } else if (admissible(rc, cc, eta)) {
      out.push_back({(int)i, (int)j, false});
    } else {
      stack.push_back({rc.Child2, cc.Child2});
      stack.push_back({rc.Child2, cc.Child1});
      stack.push_back({rc.Child1, cc.Child2});
      stack.push_back({rc.Child1, cc.Child1});
    }
  }
}

std::shared_ptr<ClusterTreeH> SpaceH::tree(int leafsize) {
  std::lock_guard<std::mutex> lk(tree_mu);
  auto it = trees.find(leafsize);
  if (it != trees.end()) return it->second;
  auto t = std::make_shared<ClusterTreeH>();
  std::unique_ptr<LevelTeam> team = make_tree_team(ndof);  // one team for both steps
  t->build(*this, leafsize, team.get());
  t->build_patches(*this, team.get());
  trees[leafsize] = t;
  return t;
}

}  // namespace bem
