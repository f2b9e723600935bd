/*
 * sgdlm_hostwrapper.hpp - the reference's C++ engine interface, restated.
 *
 * The R package's Rcpp layer (rSGDLM/src/SGDLM/RcppWrapper.cpp) reaches its
 * engine only through the abstract class SGDLM::HostWrapper<double>
 * (rSGDLM/src/SGDLM/HostWrapper.hpp:13-99) and the factory
 * SGDLM::HostWrapperFactory<double>::create (HostWrapperFactory.hpp:15-26).  This
 * header declares the same two class templates -- same namespace, same
 * virtual functions in the same order with the same parameter types -- so that
 * an object file compiled against either header calls the same vtable slots,
 * and RcppWrapper.cpp can be linked against libsgdlm_hostwrapper.so
 * (gpusgdlm_gb300/csrc/host_wrapper.cpp) in place of the reference's CUDA
 * engine.  Include one of the two headers, not both.
 *
 * Semantics are the reference's: every method is synchronous; an error (wrong
 * dimensions, wrong prior/posterior state, evolution matrices disabled, no
 * device) is logged and the call returns without effect.  Host arrays are R
 * column-major doubles; parental sets are unsigned (R's NA as 2147483648).
 */
#ifndef SGDLM_GB300_HOSTWRAPPER_HPP_
#define SGDLM_GB300_HOSTWRAPPER_HPP_

#include <cstddef>

namespace SGDLM {

template <typename DOUBLE> class HostWrapper {
 public:
  virtual ~HostWrapper() {}

  // dimensions and configuration
  virtual std::size_t getNoSeries() const = 0;
  virtual std::size_t getMaxP() const = 0;
  virtual bool getEvolutionMatrixConfiguration() const = 0;

  // device memory of the state (m series, at most max_p coefficients each)
  virtual void initMemory(std::size_t m, std::size_t max_p) = 0;
  virtual void clearMemory() = 0;
  virtual void manageEvoMemory(bool use_evolution_matrix) = 0;

  // simulation memory (draw buffers)
  virtual std::size_t getNSim() const = 0;
  virtual std::size_t getNSimBatch() const = 0;
  virtual void initSimMemory(std::size_t nsim, std::size_t nsim_batch) = 0;
  virtual void clearSimMemory() = 0;

  virtual void initForecastPriors() = 0;

  // prior/posterior flag
  virtual bool isPrior() const = 0;
  virtual void isPrior(bool prior) = 0;

  // parameters: m_t (max_p x m), C_t (max_p x max_p x m), n_t and s_t (m)
  virtual void getParameters(DOUBLE *m_t, DOUBLE *C_t, DOUBLE *n_t, DOUBLE *s_t) const = 0;
  virtual void setParameters(const DOUBLE *m_t, const DOUBLE *C_t, const DOUBLE *n_t,
                             const DOUBLE *s_t) = 0;

  // discount factors: beta (m), delta (max_p x max_p x m)
  virtual void getDiscountFactors(DOUBLE *beta, DOUBLE *delta) const = 0;
  virtual void setDiscountFactors(const DOUBLE *beta, const DOUBLE *delta) = 0;

  // evolution matrices G (max_p x max_p x m)
  virtual void getEvolutionMatrix(DOUBLE *G_t) const = 0;
  virtual void setEvolutionMatrix(const DOUBLE *G_t) = 0;

  // parental sets: p (m), sp (max_p x m)
  virtual void getParentalSets(unsigned int *p, unsigned int *sp) const = 0;
  virtual void setParentalSets(const unsigned int *p, const unsigned int *sp) = 0;

  // filtering
  virtual void computePrior(bool evolve_forecast_variables) = 0;
  virtual void computePrior(const DOUBLE *G_tp1, bool evolve_forecast_variables) = 0;
  virtual void evolveForecastSamples() = 0;
  virtual void evolveForecastSamples(const DOUBLE *G_tp1) = 0;
  virtual void computeForecast(DOUBLE *y_tp1, const DOUBLE *x_tp1, DOUBLE *lambdas,
                               DOUBLE *thetas, bool use_existing_lambdas_and_thetas) = 0;
  virtual void computePosterior(const DOUBLE *y_t, const DOUBLE *F_t) = 0;
  virtual void computeVBPosterior(DOUBLE *mean_m_t, DOUBLE *mean_C_t, DOUBLE *mean_n_t,
                                  DOUBLE *mean_s_t, DOUBLE *is_weights,
                                  DOUBLE *sum_det_weights) = 0;
};

template <typename DOUBLE> class HostWrapperFactory {
 public:
  static SGDLM::HostWrapper<DOUBLE> *create(std::size_t no_gpus);
  static SGDLM::HostWrapper<DOUBLE> *create(std::size_t no_gpus, std::size_t m, std::size_t max_p);
  static SGDLM::HostWrapper<DOUBLE> *create(std::size_t no_gpus, std::size_t m, std::size_t max_p,
                                            bool use_evolution_matrix);
};

}  // namespace SGDLM

#endif  // SGDLM_GB300_HOSTWRAPPER_HPP_
