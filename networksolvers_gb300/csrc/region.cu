// One fused two-site region step on a chain, for callers that want one library call per
// region (a Julia plugin set that hands the whole region to the device, or a C++ sweep
// driver): extracter product (extracter.jl:7), Lanczos updater (eigsolve.jl:14-28 with
// local_solvers/eigsolve.jl:3-29) and truncated-factorization inserter
// (inserter.jl:3-33).  It composes the same device pieces the separate entry points use
// (contraction engine, linear map, Lanczos, factorization), so its results are those of
// the step taken call by call.
#include "nsg_internal.h"

#include <vector>

using namespace nsg;

extern "C" {

int nsg_region_step(nsg_ctx* c, nsg_tensor* L, nsg_tensor* W1, nsg_tensor* W2, nsg_tensor* R,
                    const nsg_tensor* psi1, const nsg_tensor* psi2, int direction, int krylovdim, int maxiter,
                    double tol, double cutoff, int64_t maxdim, int64_t mindim, nsg_tensor** left,
                    nsg_tensor** right, double* energy, int64_t* newdim, double* truncerr) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && L && W1 && W2 && R && psi1 && psi2 && left && right && energy, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(direction == 0 || direction == 1, NSG_ERR_INVALID, "region_step: direction 0 or 1");
  NSG_CHECK(L->rank == 3 && R->rank == 3 && W1->rank == 4 && W2->rank == 4 && psi1->rank == 3 && psi2->rank == 3,
            NSG_ERR_INVALID, "region_step: ranks must be L 3, W1 4, W2 4, R 3, psi1 3, psi2 3");
  // labels: a, a', wl, s1, s1', wm, s2, s2', wr, b, b', c (the bond between the sites)
  enum { a = 0, ap, wl, s1, s1p, wm, s2, s2p, wr, b, bp, cb };
  // product psi1 [a, s1, c] psi2 [c, s2, b] -> local [a, s1, s2, b]
  nsg_tensor* local = nullptr;
  {
    PhaseScope phase(c, NSG_PHASE_EXTRACT);
    nsg_tensor* ts[2] = {const_cast<nsg_tensor*>(psi1), const_cast<nsg_tensor*>(psi2)};
    const int32_t labs[6] = {a, s1, cb, cb, s2, b};
    const int32_t outl[4] = {a, s1, s2, b};
    int rc = nsg_contract(c, 2, ts, labs, nullptr, 4, outl, &local);
    NSG_CHECK(rc == NSG_OK, rc, std::string("region_step: ") + c->err);
  }
  // H_eff = optimal_map(L, R, W1, W2) on [a, s1, s2, b] -> [a', s1', s2', b']
  nsg_linmap* m = nullptr;
  {
    nsg_tensor* fixed[4] = {L, R, W1, W2};
    const int32_t labs[14] = {ap, wl, a, bp, wr, b, wl, s1p, s1, wm, wm, s2p, s2, wr};
    const int32_t xl[4] = {a, s1, s2, b}, yl[4] = {ap, s1p, s2p, bp};
    int rc = nsg_linmap_create(c, 4, fixed, labs, nullptr, 4, xl, yl, &m);
    if (rc != NSG_OK) {
      nsg_tensor_release(c, local);
      throw Error(rc, std::string("region_step: ") + c->err);
    }
  }
  int numops = 0;
  int rc;
  {
    PhaseScope phase(c, NSG_PHASE_KRYLOV);
    rc = nsg_eigsolve(c, m, local, krylovdim, maxiter, tol, energy, &numops);
  }
  nsg_linmap_release(c, m);
  if (rc != NSG_OK) {
    nsg_tensor_release(c, local);
    throw Error(rc, std::string("region_step: ") + c->err);
  }
  // direction 0 (left-to-right): U [a, s1, k] -> left site, C [k, s2, b] -> right site.
  // direction 1 (right-to-left, region (v2, v1) of the plan): the factorization keeps
  // the right site's indices with U: U [s2, b, k] -> right site as [k, s2, b],
  // C [k, a, s1] -> left site as [a, s1, k].
  const int axes0[2] = {0, 1}, axes1[2] = {2, 3};
  nsg_tensor *U = nullptr, *Cf = nullptr;
  {
    PhaseScope phase(c, NSG_PHASE_FACTORIZE);
    rc = nsg_factorize(c, local, direction == 0 ? axes0 : axes1, 2, cutoff, maxdim, mindim, &U, &Cf, newdim,
                       truncerr, nullptr, 0);
  }
  nsg_tensor_release(c, local);
  NSG_CHECK(rc == NSG_OK, rc, std::string("region_step: ") + c->err);
  if (direction == 0) {
    *left = U;
    *right = Cf;
  } else {
    const int pu[3] = {2, 0, 1}, pc[3] = {1, 2, 0};
    const int64_t du[3] = {U->dims[2], U->dims[0], U->dims[1]}, dc[3] = {Cf->dims[1], Cf->dims[2], Cf->dims[0]};
    nsg_tensor* Ur = new_tensor(c, U->dtype, 3, du, false);
    nsg_tensor* Cl = new_tensor(c, Cf->dtype, 3, dc, false);
    permute(c, U, pu, false, Ur);
    permute(c, Cf, pc, false, Cl);
    free_tensor(c, U);
    free_tensor(c, Cf);
    *left = Cl;
    *right = Ur;
  }
  NSG_API_END(c)
}

}  // extern "C"
