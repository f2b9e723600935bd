// Test harness for the reference-interface adapter (tests/test_host_wrapper.py):
// drives SGDLM::HostWrapper<double> objects made by the reference's factory,
// HostWrapperFactory<double>::create, through its virtual interface only, in
// the call order of the reference's Rcpp layer (RcppWrapper.cpp).
#include <cstddef>

#include "sgdlm_hostwrapper.hpp"

using HW = SGDLM::HostWrapper<double>;
using Factory = SGDLM::HostWrapperFactory<double>;

// Construction where no device is usable: the object exists, reports empty
// dimensions and ignores calls (HostWrapperImpl.cu:19-33).  Returns 0 when so.
extern "C" int hw_no_device(void) {
  HW *w = Factory::create(1);
  if (!w) return 1;
  int bad = 0;
  bad |= w->getNoSeries() != 0;
  bad |= w->getMaxP() != 0;
  w->initMemory(4, 2);  // logged and ignored
  bad |= w->getNoSeries() != 0;
  bad |= w->getNSim() != 0;
  bad |= w->isPrior();
  bad |= w->getEvolutionMatrixConfiguration();
  delete w;
  HW *w2 = Factory::create(1, 4, 2, true);
  if (!w2) return 1;
  bad |= w2->getNoSeries() != 0;
  delete w2;
  return bad;
}

// One README time step (README.md:103-154) through the interface; outputs as
// computeVBPosterior and computeForecast write them.
extern "C" int hw_filter_step(std::size_t m, std::size_t P, const unsigned *p, const unsigned *sp,
                              const double *beta, const double *delta, const double *a,
                              const double *R, const double *r, const double *c, const double *y,
                              const double *F, const double *x, std::size_t nsim, double *om,
                              double *oC, double *on, double *os, double *ow, double *osum,
                              double *oy, int *dims_and_flags) {
  HW *w = Factory::create(1);
  if (!w) return 1;
  // setSimultaneousParents (RcppWrapper.cpp:115-120)
  if (w->getNoSeries() != m || w->getMaxP() != P) w->initMemory(m, P);
  w->setParentalSets(p, sp);
  w->setDiscountFactors(beta, delta);
  // setPriorParameters (RcppWrapper.cpp:280-282)
  w->setParameters(a, R, r, c);
  w->isPrior(true);
  dims_and_flags[0] = (int)w->getNoSeries();
  dims_and_flags[1] = (int)w->getMaxP();
  dims_and_flags[2] = w->isPrior() ? 1 : 0;
  w->computePosterior(y, F);
  dims_and_flags[3] = w->isPrior() ? 1 : 0;
  // computeVBPosterior (RcppWrapper.cpp:322-344)
  if (nsim != w->getNSim() || nsim != w->getNSimBatch()) w->initSimMemory(nsim, nsim);
  w->computeVBPosterior(om, oC, on, os, ow, osum);
  w->computePrior(false);
  dims_and_flags[4] = w->isPrior() ? 1 : 0;
  // computeForecast (RcppWrapper.cpp:442-453)
  w->initForecastPriors();
  w->computeForecast(oy, x, nullptr, nullptr, false);
  dims_and_flags[5] = (int)w->getNSim();
  // evolution matrices: disabled by default, then enabled with a round trip
  dims_and_flags[6] = w->getEvolutionMatrixConfiguration() ? 1 : 0;
  w->manageEvoMemory(true);
  dims_and_flags[7] = w->getEvolutionMatrixConfiguration() ? 1 : 0;
  delete w;
  return 0;
}
