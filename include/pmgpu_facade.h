/*
 * pmgpu_facade.h — C++ core of the ParMooN-side solver object, over the C
 * ABI of pmgpu.h only (header-only, no ParMooN headers).
 *
 * pmgpu::FgmresGPU owns one pm_handle and does what ParMooN's solver objects
 * do between TSystemNSE3D::Init and TSystemNSE3D::Solve: levels are added
 * coarsest first (TNSE_MultiGrid::AddLevel, src/FE/NSE_MultiGrid.C:81-102),
 * the first solve sets the hierarchy up (TNSE_MultiGrid::InitGPU,
 * :105-185: upload, colour, factor), and every later solve first uploads the
 * matrix values again from the caller's arrays (the caller reassembles them
 * in place between solves, as TSystemTNSE3D does every time step) unless
 * told the values are unchanged.  Iterate runs TFgmresIte::Iterate
 * (src/FE/FgmresIte.C:250-677) with the V-cycle as preconditioner and
 * returns the iteration count, as the reference's Iterate does; failures are
 * a pm_status in status() instead of the reference's exit(4711).
 *
 * pmgpu_parmoon.h wraps this class in a TItMethod for ParMooN builds.
 */
#ifndef PMGPU_FACADE_H
#define PMGPU_FACADE_H

#include <vector>

#include "pmgpu.h"

namespace pmgpu {

// The stopping parameters TItMethod keeps (include/FE/ItMethod.h:62-86).
struct StopParams {
  int restart = 20;
  int maxit = 100;
  int minit = 0;
  double red_factor = 0.0;
  double res_norm_min = 1e-10;
  double div_factor = 1e10;
};

class FgmresGPU {
 public:
  explicit FgmresGPU(const pm_options &opt) { status_ = pm_create(&h_, &opt); }
  ~FgmresGPU() {
    if (h_) pm_destroy(h_);
  }
  FgmresGPU(const FgmresGPU &) = delete;
  FgmresGPU &operator=(const FgmresGPU &) = delete;

  // Coarsest level first.  The descriptor's arrays must stay valid for the
  // lifetime of the object (their values are read again at every solve).
  pm_status AddLevel(const pm_level_desc &d) {
    if (status_ != PM_OK && !h_) return status_;
    if (setup_) return status_ = PM_BADARG;
    levels_.push_back(d);
    return status_ = pm_add_level(h_, &d);
  }

  // The caller's matrix values did not change since the last solve: the
  // next Iterate skips the upload (and the refactorisation).
  void MatricesUnchanged() { unchanged_ = true; }

  // FGMRES from the initial guess in sol; returns the iteration count, or
  // -1 when the solve could not run (status() says why).  A solve that
  // stopped at maxit or diverged returns its iterations with status()
  // PM_MAXIT / PM_DIVERGED.
  int Iterate(double *sol, const double *rhs, const StopParams &p) {
    if (!h_) return -1;
    if (!setup_) {
      status_ = pm_setup(h_);
      if (status_ != PM_OK) return -1;
      setup_ = true;
      unchanged_ = true;  // pm_setup has just read the values
    }
    if (!unchanged_) {
      status_ = pm_update_matrices(h_, levels_.data(), (int)levels_.size());
      if (status_ != PM_OK) return -1;
    }
    unchanged_ = false;
    status_ = pm_set_tolerances(h_, p.restart, p.maxit, p.minit, p.red_factor, p.res_norm_min,
                                p.div_factor);
    if (status_ != PM_OK) return -1;
    status_ = pm_solve(h_, sol, rhs, &result_);
    if (status_ != PM_OK && status_ != PM_MAXIT && status_ != PM_DIVERGED) return -1;
    return result_.iterations;
  }

  pm_status status() const { return status_; }
  const pm_result &result() const { return result_; }
  const char *error() const { return h_ ? pm_last_error(h_) : pm_status_string(status_); }
  pm_handle *handle() { return h_; }

 private:
  pm_handle *h_ = nullptr;
  pm_status status_ = PM_OK;
  std::vector<pm_level_desc> levels_;
  bool setup_ = false, unchanged_ = false;
  pm_result result_ = {};
};

}  // namespace pmgpu

#endif  // PMGPU_FACADE_H
