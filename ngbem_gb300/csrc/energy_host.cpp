// Host side of the batched single-layer energy (energy.cu): topology tables built once per
// batch, then any number of evaluations for new vertex coordinates and densities.
#include <algorithm>

#include "host.hpp"

namespace bem {

void SLBatch::build(int nprob_, const int* nverts, const int* ntris, const int* tris, int order_reg, int order_sing,
                    int prec_, int dual_) {
  if (nprob_ < 1) throw Error(BEM_ERR_ARG, "at least one problem");
  if (order_reg < 0 || order_reg > 5) throw Error(BEM_ERR_ARG, "regular order must be in 0..5");
  if (order_sing < 0 || order_sing > 12) throw Error(BEM_ERR_ARG, "singular order must be in 0..12");
  nprob = nprob_;
  prec = prec_;
  dual = dual_;
  std::vector<int> t0(nprob), nt(nprob), v0(nprob);
  for (int b = 0; b < nprob; ++b) {
    if (nverts[b] < 3 || ntris[b] < 1) throw Error(BEM_ERR_ARG, "empty mesh in the batch");
    t0[b] = ntri;
    nt[b] = ntris[b];
    v0[b] = nvert;
    ntri += ntris[b];
    nvert += nverts[b];
  }
  std::vector<int4> tri(ntri);
  std::vector<int> tprob(ntri);
  for (int b = 0; b < nprob; ++b)
    for (int e = 0; e < nt[b]; ++e) {
      const int* t = tris + 3 * (size_t)(t0[b] + e);
      for (int k = 0; k < 3; ++k)
        if (t[k] < 0 || t[k] >= nverts[b]) throw Error(BEM_ERR_ARG, "vertex index out of range");
      tri[t0[b] + e] = make_int4(v0[b] + t[0], v0[b] + t[1], v0[b] + t[2], 0);
      tprob[t0[b] + e] = b;
    }
  // ordered element pairs sharing at least one vertex (identical pairs included)
  std::vector<int2> sing;
  {
    std::vector<std::vector<int>> vt(nvert);
    for (int e = 0; e < ntri; ++e) {
      vt[tri[e].x].push_back(e);
      vt[tri[e].y].push_back(e);
      vt[tri[e].z].push_back(e);
    }
    std::vector<int> nb;
    for (int e = 0; e < ntri; ++e) {
      nb.clear();
      for (int v : {tri[e].x, tri[e].y, tri[e].z})
        for (int f : vt[v]) nb.push_back(f);
      std::sort(nb.begin(), nb.end());
      nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
      for (int f : nb) sing.push_back(make_int2(e, f));
    }
  }
  // work units of the regular kernel, the largest problems first
  const TrigRule r = make_trig_rule(order_reg);
  nq = (int)r.w.size();
  const int ti = sle_tile_test(), tj = sle_tile_trial(prec == 0, nq);
  std::vector<int> order(nprob);
  for (int b = 0; b < nprob; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return nt[x] > nt[y]; });
  std::vector<int4> units;
  for (int b : order)
    for (int i0 = 0; i0 < nt[b]; i0 += ti)
      for (int j0 = 0; j0 < nt[b]; j0 += tj) units.push_back(make_int4(b, i0, j0, 0));
  for (int q = 0; q < nq; ++q) {
    rxi[q] = r.xi[q];
    reta[q] = r.eta[q];
    rw[q] = r.w[q];
  }
  for (int c = 0; c < 3; ++c) {
    // one point per direction (the Laplace kernel's homogeneity sums the radial points)
    SSRule s = make_ss_rule(c, order_sing, true);
    ss_n[c] = (int)s.w.size();
    ss_c1 = s.c1;
    ss_c2 = s.c2;
    std::vector<double> tab;
    tab.insert(tab.end(), s.x0.begin(), s.x0.end());
    tab.insert(tab.end(), s.x1.begin(), s.x1.end());
    tab.insert(tab.end(), s.y0.begin(), s.y0.end());
    tab.insert(tab.end(), s.y1.begin(), s.y1.end());
    tab.insert(tab.end(), s.w.begin(), s.w.end());
    d_ss[c].upload(tab);
  }
  d_tri.upload(tri);
  d_tprob.upload(tprob);
  d_t0.upload(t0);
  d_nt.upload(nt);
  d_units.upload(units);
  d_sing.upload(sing);
  nunits = (int)units.size();
  nsing = (int)sing.size();
  d_D.alloc((size_t)ntri * sizeof(double));
  d_dD.alloc((size_t)ntri * 9 * sizeof(double));
  d_cf.alloc((size_t)ntri * 6 * sizeof(float));
  d_off.alloc((size_t)ntri * nq * 3 * sizeof(float));
  d_q64.alloc((size_t)ntri * nq * 3 * sizeof(double));
  long long reg = 0;
  for (int b = 0; b < nprob; ++b) reg += (long long)nt[b] * nt[b];
  npairs_regular = reg - nsing;
  BEM_CUDA(cudaDeviceSynchronize());
}

void SLBatch::eval(const double* X, const double* u, const double* wprob, double* energy, double* vu, double* grad,
                   cudaStream_t s) {
  if (!X || !u) throw Error(BEM_ERR_ARG, "null coordinates or densities");
  // outputs that the caller does not want still need somewhere to accumulate
  if (!energy || !vu) {
    if (scratch_out.bytes < (size_t)(nprob + ntri) * sizeof(double)) scratch_out.alloc((size_t)(nprob + ntri) * sizeof(double));
    if (!energy) energy = scratch_out.as<double>();
    if (!vu) vu = scratch_out.as<double>() + nprob;
  }
  BEM_CUDA(cudaMemsetAsync(energy, 0, (size_t)nprob * sizeof(double), s));
  BEM_CUDA(cudaMemsetAsync(vu, 0, (size_t)ntri * sizeof(double), s));
  if (grad) BEM_CUDA(cudaMemsetAsync(grad, 0, (size_t)nvert * 3 * sizeof(double), s));
  SLEArgs a{};
  a.X = X;
  a.tri = d_tri.as<int4>();
  a.u = u;
  a.wprob = wprob;
  a.tprob = d_tprob.as<int>();
  a.t0 = d_t0.as<int>();
  a.nt = d_nt.as<int>();
  a.ntri = ntri;
  a.dual = dual;
  a.nq = nq;
  for (int q = 0; q < nq; ++q) {
    a.rxi[q] = rxi[q];
    a.reta[q] = reta[q];
    a.rw[q] = rw[q];
  }
  a.D = d_D.as<double>();
  a.dD = d_dD.as<double>();
  a.cf = d_cf.as<float>();
  a.off = d_off.as<float>();
  a.q64 = d_q64.as<double>();
  a.units = d_units.as<int4>();
  a.nunits = nunits;
  a.sing = d_sing.as<int2>();
  a.nsing = nsing;
  for (int c = 0; c < 3; ++c) {
    a.ss[c] = d_ss[c].as<double>();
    a.ss_n[c] = ss_n[c];
  }
  a.ss_smem = 40 * (ss_n[0] + ss_n[1] + ss_n[2]) <= 48 * 1024 ? 1 : 0;
  a.ss_c1 = ss_c1;
  a.ss_c2 = ss_c2;
  a.energy = energy;
  a.vu = vu;
  a.grad = grad;
  launch_sle(a, prec == 0, grad != nullptr, s);
  BEM_CUDA(cudaGetLastError());
}

}  // namespace bem
