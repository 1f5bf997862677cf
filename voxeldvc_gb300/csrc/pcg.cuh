// Device-resident state of one preconditioned CG solve.  Every PCG kernel
// reads `done` first and returns without touching memory once it is set, so
// a captured chunk of iterations can be replayed past convergence safely.
#pragma once

namespace vdvc {

struct PcgState {
  double rz;     // r . z of the current iterate
  double r0;     // b . b + 1e-30
  double alpha;  // step of the current iteration
  double beta;   // p <- z + beta p for the next iteration
  double res;    // sqrt(r.r / r0) after the last update
  double rr;     // r . r after the last update
  int iter;      // completed iterations
  int done;      // 1 once converged or max_iter reached
  int status;    // VDVC_OK, VDVC_ERR_NONFINITE
  int max_iter;
  double tol;
};

}  // namespace vdvc
