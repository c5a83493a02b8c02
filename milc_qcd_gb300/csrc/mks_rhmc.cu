// mks_rhmc.cu -- one RHMC trajectory on the GPU, MILC's update().
//
// Sequences the device-resident pieces exactly as
// ks_imp_rhmc/update_rhmc.c:update() does for the HISQ action:
//   ranmom                       generic/ranmom.c
//   grsource_imp_rhmc            ks_imp_rhmc/grsource_rhmc.c:17-50 (per field)
//   d_action_rhmc                ks_imp_rhmc/d_action_rhmc.c:17-86
//   integrators                  update_rhmc.c:263-473 (leapfrog, Omelyan,
//                                2G1F, 3G1F), reunitarize_ks after each
//                                (double) step
//   update_h_gauge / _fermion    ks_imp_rhmc/update_h_rhmc.c:16-105
//   ks_ratinv / ks_rateval       ks_imp_rhmc/ks_ratinv.c:29-137
// Thin links, momenta, pseudofermion fields and every solution vector stay
// on the device for the whole trajectory; the host only steers (solver
// polling, scalar results).  No accept/reject: the caller decides with
// delta_s (MILC draws its Metropolis number from node_prn).
#include <chrono>
#include <cstring>
#include <vector>
#include "mks_internal.cuh"

namespace mks {

namespace {

double wall() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Traj {
  const mks_rhmc_params *p;
  mks_rhmc_result *r;
  std::vector<double> eps_distinct;
  std::vector<int> inaik;          // Naik group of each field
  double *phi = nullptr;           // [n_pseudo][V][6]
  double *xs = nullptr;            // [max_terms][V][6] solutions (AoS)
  double *tmp = nullptr;           // [V][6]
  double *gtmp = nullptr;          // [n_pseudo][V][6] heat-bath Gaussians
  float2 *xs32 = nullptr;          // [terms][2][3][Vh] force input, FP32 setting
  double2 *xs_soa = nullptr;       // [max_terms][2][3][Vh] force input
  int max_terms = 0;

  size_t vsz() const { return ctx().V * 6; }
  double *phi_of(int i) const { return phi + (size_t)i * vsz(); }
  double *x_of(int j) const { return xs + (size_t)j * vsz(); }

  int links() {
    Context &c = ctx();
    if (c.slots[0].valid && c.aux_action == MKS_ACTION_HISQ && c.links_prec == c.md_prec) return MKS_OK;
    const double t0 = wall();
    MKS_TRY(links_from_aux(MKS_ACTION_HISQ, (int)eps_distinct.size(), eps_distinct.data(), 1.0));
    r->t_links += wall() - t0;
    return MKS_OK;
  }

  const mks_ratfunc &fn(int ipf, int tag) const {
    const mks_pseudofermion &f = p->pf[ipf];
    return tag == 0 ? f.md : (tag == 1 ? f.gr : f.fa);
  }
  double resid(int ipf, int tag) const {
    const mks_pseudofermion &f = p->pf[ipf];
    return tag == 0 ? f.resid_md : (tag == 1 ? f.resid_gr : f.resid_fa);
  }
  int prec(int tag) const { return tag == 0 ? p->prec_md : (tag == 1 ? p->prec_gr : p->prec_fa); }

  // psim_j = (pole_{j+1} - D_eo D_oe)^-1 src on even sites, j < order, into xs[x0 ...]
  int ratinv(const double *src, int ipf, int tag, int x0) {
    MKS_TRY(links());
    const mks_ratfunc &f = fn(ipf, tag);
    const int order = f.order;
    std::vector<double *> psim(order);
    for (int j = 0; j < order; j++) {
      psim[j] = x_of(x0 + j);
      MKS_CUDA(cudaMemsetAsync(psim[j], 0, vsz() * sizeof(double), ctx().stream));
    }
    mks_invert_arg arg;
    arg.max = p->pf[ipf].max_cg;
    arg.nrestart = p->nrestart > 0 ? p->nrestart : 5;
    arg.parity = MKS_EVEN;
    arg.prec = prec(tag);
    arg.resid = resid(ipf, tag);
    arg.relresid = 0.0;
    arg.delta = 0.1;
    std::vector<mks_invert_result> res(order);
    const double t0 = wall();
    const int it = mks_ks_multicg_offset_field_dev(src, psim.data(), f.pole + 1, order, inaik[ipf], &arg,
                                                   res.data());
    r->t_solve += wall() - t0;
    if (it < 0) return it;
    for (int j = 0; j < order; j++)
      if (!res[j].converged) r->unconverged++;
    r->cg_iters += it;
    r->n_solves++;
    return MKS_OK;
  }

  // fields of Naik group g (they share the links of slot g), in field order
  std::vector<int> group(int g) const {
    std::vector<int> fs;
    for (int i = 0; i < p->n_pseudo; i++)
      if (inaik[i] == g) fs.push_back(i);
    return fs;
  }

  // ratinv for the fields fs of one Naik group (sources srcs[k], psim of
  // field fs[k] into xs from x0[k] on).  In FP32 with equal residuals and
  // iteration caps the fields' multi-shift solves run batched (one
  // multi-source D_eo pair per iteration for all of them); otherwise one
  // field after the other.
  int ratinv_many(const std::vector<int> &fs, int tag, const std::vector<const double *> &srcs,
                  const std::vector<int> &x0) {
    bool batch = fs.size() >= 2 && fs.size() <= 4 && prec(tag) == MKS_PREC_SINGLE;
    for (size_t k = 1; k < fs.size() && batch; k++)
      batch = resid(fs[k], tag) == resid(fs[0], tag) && p->pf[fs[k]].max_cg == p->pf[fs[0]].max_cg;
    if (!batch) {
      for (size_t k = 0; k < fs.size(); k++) MKS_TRY(ratinv(srcs[k], fs[k], tag, x0[k]));
      return MKS_OK;
    }
    MKS_TRY(links());
    std::vector<int> ns;
    std::vector<double> offs;
    std::vector<double *> psim;
    for (size_t k = 0; k < fs.size(); k++) {
      const mks_ratfunc &f = fn(fs[k], tag);
      ns.push_back(f.order);
      for (int j = 0; j < f.order; j++) {
        offs.push_back(f.pole[j + 1]);
        psim.push_back(x_of(x0[k] + j));
        MKS_CUDA(cudaMemsetAsync(psim.back(), 0, vsz() * sizeof(double), ctx().stream));
      }
    }
    mks_invert_arg arg;
    arg.max = p->pf[fs[0]].max_cg;
    arg.nrestart = p->nrestart > 0 ? p->nrestart : 5;
    arg.parity = MKS_EVEN;
    arg.prec = prec(tag);
    arg.resid = resid(fs[0], tag);
    arg.relresid = 0.0;
    arg.delta = 0.1;
    std::vector<mks_invert_result> res(offs.size());
    const double t0 = wall();
    const int it = mks_ks_multicg_offset_multi_dev((int)fs.size(), srcs.data(), ns.data(), offs.data(), psim.data(),
                                                   inaik[fs[0]], &arg, res.data());
    r->t_solve += wall() - t0;
    if (it < 0) return it;
    for (const mks_invert_result &q : res)
      if (!q.converged) r->unconverged++;
    r->cg_iters += it;
    r->n_solves += (int)fs.size();
    return MKS_OK;
  }

  // out = res_0 src + sum_j res_{j+1} psim_j on even sites
  int rateval(const double *src, int ipf, int tag, int x0, double *out) {
    const mks_ratfunc &f = fn(ipf, tag);
    std::vector<const double *> x(f.order);
    for (int j = 0; j < f.order; j++) x[j] = x_of(x0 + j);
    return lincomb_aos_dev(0, src, x.data(), f.res, f.order, out);
  }

  // grsource_rhmc.c: the Gaussians of all fields are drawn first, in field
  // order (the solves use no random numbers, so the sequence is MILC's)
  int grsource() {
    Context &c = ctx();
    for (int ipf = 0; ipf < p->n_pseudo; ipf++) {
      double *g = gtmp + (size_t)ipf * vsz();
      MKS_CUDA(cudaMemsetAsync(g, 0, vsz() * sizeof(double), c.stream));
      MKS_TRY(gauss_vec_dev(MKS_EVEN, g));
      if (ipf < MKS_RHMC_MAX_PSEUDO) MKS_TRY(norm2_aos_dev(g, 0, &r->grsource_sum[ipf]));
    }
    for (int gi = 0; gi < (int)eps_distinct.size(); gi++) {
      const std::vector<int> fs = group(gi);
      std::vector<const double *> srcs;
      std::vector<int> x0;
      int off = 0;
      for (int f : fs) {
        srcs.push_back(gtmp + (size_t)f * vsz());
        x0.push_back(off);
        off += fn(f, 1).order;
      }
      MKS_TRY(ratinv_many(fs, 1, srcs, x0));
      for (size_t k = 0; k < fs.size(); k++) {
        MKS_CUDA(cudaMemsetAsync(phi_of(fs[k]), 0, vsz() * sizeof(double), c.stream));
        MKS_TRY(rateval(srcs[k], fs[k], 1, x0[k], phi_of(fs[k])));
      }
    }
    return MKS_OK;
  }

  int action(double *g, double *h, double *f) {
    MKS_TRY(gauge_action_dev(p->beta, p->u0, p->nflavors, g));
    MKS_TRY(mom_action_dev(h));
    std::vector<double> sf(p->n_pseudo, 0.0);
    for (int gi = 0; gi < (int)eps_distinct.size(); gi++) {
      const std::vector<int> fs = group(gi);
      std::vector<const double *> srcs;
      std::vector<int> x0;
      int off = 0;
      for (int fi : fs) {
        srcs.push_back(phi_of(fi));
        x0.push_back(off);
        off += fn(fi, 2).order;
      }
      MKS_TRY(ratinv_many(fs, 2, srcs, x0));
      for (size_t k = 0; k < fs.size(); k++) {
        MKS_TRY(rateval(phi_of(fs[k]), fs[k], 2, x0[k], tmp));
        MKS_TRY(norm2_aos_dev(tmp, 0, &sf[fs[k]]));
      }
    }
    *f = 0.0;
    for (int ipf = 0; ipf < p->n_pseudo; ipf++) *f += sf[ipf];   // field order
    return MKS_OK;
  }

  int update_u(double eps) { return update_u_dev(eps); }

  int update_h_gauge(double eps) {
    const double t0 = wall();
    MKS_TRY(gauge_force_dev(eps, p->beta, p->u0, p->nflavors, ctx().md_prec));
    MKS_CUDA(cudaStreamSynchronize(ctx().stream));
    r->t_gauge_force += wall() - t0;
    r->n_gauge_force++;
    return MKS_OK;
  }

  // update_h_rhmc.c:40-105: X_j = (M^dag M + pole)^-1 phi on even sites,
  // D_oe X_j on odd sites, all fields grouped by Naik epsilon, one force call.
  // In the FP32 molecular-dynamics setting the solutions go to FP32 and
  // D_oe X_j is applied in FP32 (multi-source, the slot's FP32 links) --
  // the force that consumes them computes in FP32 -- else in FP64 as MILC.
  int update_h_fermion(double eps) {
    Context &c = ctx();
    MKS_TRY(links());
    const int n_naiks = (int)eps_distinct.size();
    const bool low = c.md_prec == MKS_PREC_SINGLE;
    std::vector<int> orders(n_naiks, 0);
    std::vector<double> allres;
    int t = 0;
    double t_doe = 0.0;
    for (int g = 0; g < n_naiks; g++) {
      const std::vector<int> fs = group(g);
      std::vector<const double *> srcs;
      std::vector<int> x0;
      int off = t;
      for (int ipf : fs) {
        srcs.push_back(phi_of(ipf));
        x0.push_back(off);
        off += fn(ipf, 0).order;
      }
      MKS_TRY(ratinv_many(fs, 0, srcs, x0));
      const double td = wall();
      const int tg = t;
      for (int ipf : fs) {
        const mks_ratfunc &f = fn(ipf, 0);
        for (int j = 0; j < f.order; j++) {
          if (!low) MKS_TRY(mks_dslash_fn_field_dev(x_of(t + j), x_of(t + j), MKS_ODD, g));
          allres.push_back(f.res[j + 1]);
        }
        orders[g] += f.order;
        t += f.order;
      }
      if (low) {
        std::vector<float2 *> ev, od;
        for (int j = tg; j < t; j++) {
          float2 *x = xs32 + (size_t)j * 6 * c.Vh;
          MKS_TRY(vec_aos_to_soa32(x_of(j), x, 0));
          ev.push_back(x);
          od.push_back(x + 3 * c.Vh);
        }
        MKS_TRY(dslash32_multi(g, 1, t - tg, ev.data(), od.data()));
      }
      t_doe += wall() - td;
    }
    const double t0 = wall();
    if (low) {
      std::vector<float2 *> xp(t);
      for (int j = 0; j < t; j++) xp[j] = xs32 + (size_t)j * 6 * c.Vh;
      MKS_TRY(force_dev32(eps, allres.data(), xp.data(), t, orders.data(), n_naiks, c.mom));
    } else {
      std::vector<double2 *> xp(t);
      for (int j = 0; j < t; j++) {
        xp[j] = xs_soa + (size_t)j * 6 * c.Vh;
        MKS_TRY(vec_aos_to_soa64(x_of(j), xp[j], 0));
        MKS_TRY(vec_aos_to_soa64(x_of(j), xp[j] + 3 * c.Vh, 1));
      }
      MKS_TRY(force_dev(eps, allres.data(), xp.data(), t, orders.data(), n_naiks, c.mom, nullptr));
    }
    r->t_fermion_force += wall() - t0 + t_doe;
    r->n_fermion_force++;
    return MKS_OK;
  }

  int update_h_rhmc(double eps) {
    MKS_TRY(update_h_gauge(eps));
    return update_h_fermion(eps);
  }

  int reunit() { return reunitarize_dev(); }

  // update_rhmc.c:263-473
  int integrate() {
    const double eps = p->epsilon;
    const int steps = p->steps;
    switch (p->int_alg) {
    case MKS_INT_LEAPFROG:
      for (int s = 1; s <= steps; s++) {
        MKS_TRY(update_u(0.5 * eps));
        MKS_TRY(update_h_rhmc(eps));
        MKS_TRY(update_u(0.5 * eps));
        MKS_TRY(reunit());
      }
      return MKS_OK;
    case MKS_INT_OMELYAN: {
      const double lambda = 0.8;
      if (steps % 2) return MKS_ERR_ARG;
      for (int s = 2; s <= steps; s += 2) {
        MKS_TRY(update_u(0.5 * eps * lambda));
        MKS_TRY(update_h_rhmc(eps));
        MKS_TRY(update_u(eps * (2.0 - lambda)));
        MKS_TRY(update_h_rhmc(eps));
        MKS_TRY(update_u(0.5 * eps * lambda));
        MKS_TRY(reunit());
      }
      return MKS_OK;
    }
    case MKS_INT_2G1F: {
      const double alpha = 0.1, beta = 0.1;
      if (steps % 2) return MKS_ERR_ARG;
      const double tu[7] = {0.25 - 0.5 * alpha, 0.5 - beta, 0.75 + 0.5 * alpha, 1.25 - 0.5 * alpha, 1.5 + beta,
                            1.75 + 0.5 * alpha, 2.0};
      const char kick[7] = {'G', 'F', 'G', 'G', 'F', 'G', 0};
      for (int s = 2; s <= steps; s += 2) {
        double prev = 0.0;
        for (int k = 0; k < 7; k++) {
          MKS_TRY(update_u(eps * (tu[k] - prev)));
          prev = tu[k];
          if (kick[k] == 'G') MKS_TRY(update_h_gauge(0.5 * eps));
          if (kick[k] == 'F') MKS_TRY(update_h_fermion(eps));
        }
        MKS_TRY(reunit());
      }
      return MKS_OK;
    }
    case MKS_INT_3G1F: {
      const double alpha = 0.1, beta = 0.1;
      if (steps % 2) return MKS_ERR_ARG;
      const double tu[9] = {1.0 / 6.0 - alpha / 3.0, 0.5 - beta, 3.0 / 6.0 + alpha / 3.0, 5.0 / 6.0 - alpha / 3.0,
                            7.0 / 6.0 + alpha / 3.0, 9.0 / 6.0 - alpha / 3.0, 1.5 + beta, 11.0 / 6.0 + alpha / 3.0,
                            2.0};
      const char kick[9] = {'G', 'F', 'G', 'G', 'G', 'G', 'F', 'G', 0};
      for (int s = 2; s <= steps; s += 2) {
        double prev = 0.0;
        for (int k = 0; k < 9; k++) {
          MKS_TRY(update_u(eps * (tu[k] - prev)));
          prev = tu[k];
          if (kick[k] == 'G') MKS_TRY(update_h_gauge(eps / 3.0));
          if (kick[k] == 'F') MKS_TRY(update_h_fermion(eps));
        }
        MKS_TRY(reunit());
      }
      return MKS_OK;
    }
    default:
      return MKS_ERR_ARG;
    }
  }

  int run() {
    Context &c = ctx();
    const double t0 = wall();
    if (p->refresh) {
      MKS_TRY(ranmom_dev());
      MKS_TRY(grsource());
    }
    MKS_TRY(action(&r->g0, &r->h0, &r->f0));
    // forces and the links rebuilt for them in the arithmetic asked for;
    // the action before and after is always evaluated in FP64
    c.md_prec = p->prec_force == MKS_PREC_SINGLE ? MKS_PREC_SINGLE : MKS_PREC_DOUBLE;
    int rc = integrate();
    c.md_prec = MKS_PREC_DOUBLE;
    MKS_TRY(rc);
    MKS_TRY(action(&r->g1, &r->h1, &r->f1));
    r->delta_s = (r->g1 + r->h1 + r->f1) - (r->g0 + r->h0 + r->f0);
    MKS_TRY(plaquette_dev(&r->plaq_ss, &r->plaq_st));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    r->t_total = wall() - t0;
    return MKS_OK;
  }
};

// pseudofermion fields persist between trajectories (refresh = 0 reuses them)
double *g_phi = nullptr;
size_t g_phi_bytes = 0;

}  // namespace

void rhmc_free() {
  dev_free(g_phi);
  g_phi = nullptr;
  g_phi_bytes = 0;
}

}  // namespace mks

using namespace mks;

extern "C" {

int mks_rhmc_trajectory(const mks_rhmc_params *p, mks_rhmc_result *r) {
  MKS_TRY(check_ready());
  if (!p || !r || !p->pf || p->n_pseudo < 1 || p->n_pseudo > MKS_RHMC_MAX_PSEUDO) return MKS_ERR_ARG;
  if (!(p->u0 > 0) || p->steps < 1 || p->nflavors < 0) return MKS_ERR_ARG;
  Context &c = ctx();
  if (!c.auxU || !c.mom) return MKS_ERR_STATE;
  memset(r, 0, sizeof *r);
  Traj T;
  T.p = p;
  T.r = r;
  int total = 0, maxo = 0, total_gr = 0, total_fa = 0;
  for (int i = 0; i < p->n_pseudo; i++) {
    const mks_pseudofermion &f = p->pf[i];
    const mks_ratfunc *fs[3] = {&f.md, &f.gr, &f.fa};
    for (const mks_ratfunc *q : fs) {
      if (q->order < 1 || q->order > 32 || !q->res || !q->pole) return MKS_ERR_ARG;
      for (int j = 1; j <= q->order; j++)
        if (!(q->pole[j] > 0)) return MKS_ERR_ARG;
      maxo = q->order > maxo ? q->order : maxo;
    }
    if (f.max_cg < 1 || !(f.resid_md > 0) || !(f.resid_fa > 0) || !(f.resid_gr > 0)) return MKS_ERR_ARG;
    total += f.md.order;
    total_gr += f.gr.order;
    total_fa += f.fa.order;
    int g = -1;
    for (size_t k = 0; k < T.eps_distinct.size(); k++)
      if (T.eps_distinct[k] == f.naik_eps) g = (int)k;
    if (g < 0) {
      if ((int)T.eps_distinct.size() >= MKS_MAX_SLOTS) return MKS_ERR_ARG;
      g = (int)T.eps_distinct.size();
      T.eps_distinct.push_back(f.naik_eps);
    }
    T.inaik.push_back(g);
  }
  if (T.eps_distinct[0] != 0.0) return MKS_ERR_ARG;  // MILC: the first Naik group has epsilon 0
  if (total > 64) return MKS_ERR_ARG;               // force terms per call
  T.max_terms = total > maxo ? total : maxo;
  T.max_terms = total_gr > T.max_terms ? total_gr : T.max_terms;   // a Naik group's fields solved together
  T.max_terms = total_fa > T.max_terms ? total_fa : T.max_terms;
  const size_t vb = c.V * 6 * sizeof(double);
  const size_t phi_bytes = (size_t)p->n_pseudo * vb;
  if (!p->refresh && (!g_phi || g_phi_bytes != phi_bytes)) return MKS_ERR_STATE;
  if (g_phi_bytes != phi_bytes) {
    rhmc_free();
    MKS_TRY(dev_alloc((void **)&g_phi, phi_bytes));
    g_phi_bytes = phi_bytes;
  }
  T.phi = g_phi;
  int rc = dev_alloc((void **)&T.xs, (size_t)T.max_terms * vb);
  if (rc >= 0) rc = dev_alloc((void **)&T.tmp, vb);
  if (rc >= 0) rc = dev_alloc((void **)&T.gtmp, (size_t)p->n_pseudo * vb);
  if (rc >= 0) rc = dev_alloc((void **)&T.xs_soa, (size_t)total * 6 * c.Vh * sizeof(double2));
  if (rc >= 0 && p->prec_force == MKS_PREC_SINGLE)
    rc = dev_alloc((void **)&T.xs32, (size_t)total * 6 * c.Vh * sizeof(float2));
  if (rc >= 0) rc = T.run();
  dev_free(T.xs);
  dev_free(T.tmp);
  dev_free(T.gtmp);
  dev_free(T.xs_soa);
  dev_free(T.xs32);
  return rc;
}

}  // extern "C"
