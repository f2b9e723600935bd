// SGDLM::HostWrapper<double> on the GB300 engine: the drop-in for the
// reference's SGDLM::HostWrapperImpl<double> (rSGDLM/src/SGDLM/HostWrapperImpl.cu)
// behind the reference's own factory, HostWrapperFactory<double>::create
// (HostWrapperFactory.cu:5-35).  Each virtual forwards to one entry point of
// include/sgdlm.h; the C functions log an error and leave the state unchanged
// where the reference logs and returns (myAssert, rSGDLM/src/logger.hpp:160-165),
// so the void methods here return after the call whatever its status.
//
// Built as libsgdlm_hostwrapper.so (g++, no CUDA headers), linked against
// libsgdlm_gb300.so.  Compiled with -DSGDLM_USE_REFERENCE_HEADERS and the
// reference's source directory on the include path, it builds against the
// reference's own HostWrapper.hpp / HostWrapperFactory.hpp instead of
// include/sgdlm_hostwrapper.hpp (the interface check of the tests).
#include <cstddef>
#include <cstdio>

#ifdef SGDLM_USE_REFERENCE_HEADERS
#include "SGDLM/HostWrapper.hpp"
#include "SGDLM/HostWrapperFactory.hpp"
#else
#include "../../include/sgdlm_hostwrapper.hpp"
#endif
#include "../../include/sgdlm.h"

namespace {

class GB300HostWrapper final : public SGDLM::HostWrapper<double> {
 public:
  explicit GB300HostWrapper(std::size_t no_gpus) {
    // HostWrapperImpl.cu:19-33: with no device the reference logs and keeps an
    // engine of zero GPUs, whose every call does nothing
    if (sgdlm_create(no_gpus, &h_) != SGDLM_OK) {
      h_ = nullptr;
      std::fprintf(stderr, "Error: No cuda-enabled devices available.\n");
    }
  }
  ~GB300HostWrapper() override { sgdlm_destroy(h_); }
  GB300HostWrapper(const GB300HostWrapper &) = delete;
  GB300HostWrapper &operator=(const GB300HostWrapper &) = delete;

  std::size_t getNoSeries() const override {
    std::size_t v = 0;
    if (h_) sgdlm_get_no_series(h_, &v);
    return v;
  }
  std::size_t getMaxP() const override {
    std::size_t v = 0;
    if (h_) sgdlm_get_max_p(h_, &v);
    return v;
  }
  bool getEvolutionMatrixConfiguration() const override {
    int v = 0;
    if (h_) sgdlm_get_evolution_matrix_configuration(h_, &v);
    return v != 0;
  }

  void initMemory(std::size_t m, std::size_t max_p) override {
    if (h_) sgdlm_init_memory(h_, m, max_p);
  }
  void clearMemory() override {
    if (h_) sgdlm_clear_memory(h_);
  }
  void manageEvoMemory(bool use) override {
    if (h_) sgdlm_manage_evo_memory(h_, use ? 1 : 0);
  }

  std::size_t getNSim() const override {
    std::size_t v = 0;
    if (h_) sgdlm_get_nsim(h_, &v);
    return v;
  }
  std::size_t getNSimBatch() const override {
    std::size_t v = 0;
    if (h_) sgdlm_get_nsim_batch(h_, &v);
    return v;
  }
  void initSimMemory(std::size_t nsim, std::size_t nsim_batch) override {
    if (h_) sgdlm_init_sim_memory(h_, nsim, nsim_batch);
  }
  void clearSimMemory() override {
    if (h_) sgdlm_clear_sim_memory(h_);
  }
  void initForecastPriors() override {
    if (h_) sgdlm_init_forecast_priors(h_);
  }

  bool isPrior() const override {
    int v = 0;
    if (h_) sgdlm_is_prior(h_, &v);
    return v != 0;
  }
  void isPrior(bool prior) override {
    if (h_) sgdlm_set_is_prior(h_, prior ? 1 : 0);
  }

  void getParameters(double *m_t, double *C_t, double *n_t, double *s_t) const override {
    if (h_) sgdlm_get_parameters(h_, m_t, C_t, n_t, s_t);
  }
  void setParameters(const double *m_t, const double *C_t, const double *n_t,
                     const double *s_t) override {
    if (h_) sgdlm_set_parameters(h_, m_t, C_t, n_t, s_t);
  }
  void getDiscountFactors(double *beta, double *delta) const override {
    if (h_) sgdlm_get_discount_factors(h_, beta, delta);
  }
  void setDiscountFactors(const double *beta, const double *delta) override {
    if (h_) sgdlm_set_discount_factors(h_, beta, delta);
  }
  void getEvolutionMatrix(double *G_t) const override {
    if (h_) sgdlm_get_evolution_matrix(h_, G_t);
  }
  void setEvolutionMatrix(const double *G_t) override {
    if (h_) sgdlm_set_evolution_matrix(h_, G_t);
  }
  void getParentalSets(unsigned int *p, unsigned int *sp) const override {
    if (h_) sgdlm_get_parental_sets(h_, p, sp);
  }
  void setParentalSets(const unsigned int *p, const unsigned int *sp) override {
    if (h_) sgdlm_set_parental_sets(h_, p, sp);
  }

  void computePrior(bool evolve_forecast_variables) override {
    if (h_) sgdlm_compute_prior(h_, evolve_forecast_variables ? 1 : 0);
  }
  void computePrior(const double *G_tp1, bool evolve_forecast_variables) override {
    if (h_) sgdlm_compute_evo_prior(h_, G_tp1, evolve_forecast_variables ? 1 : 0);
  }
  void evolveForecastSamples() override {
    if (h_) sgdlm_evolve_forecast_samples(h_);
  }
  void evolveForecastSamples(const double *G_tp1) override {
    if (h_) sgdlm_evolve_forecast_samples_evo(h_, G_tp1);
  }
  void computeForecast(double *y_tp1, const double *x_tp1, double *lambdas, double *thetas,
                       bool use_existing_lambdas_and_thetas) override {
    if (h_)
      sgdlm_compute_forecast(h_, y_tp1, x_tp1, lambdas, thetas,
                             use_existing_lambdas_and_thetas ? 1 : 0);
  }
  void computePosterior(const double *y_t, const double *F_t) override {
    if (h_) sgdlm_compute_posterior(h_, y_t, F_t);
  }
  void computeVBPosterior(double *mean_m_t, double *mean_C_t, double *mean_n_t,
                          double *mean_s_t, double *is_weights,
                          double *sum_det_weights) override {
    if (h_)
      sgdlm_compute_vb_posterior(h_, mean_m_t, mean_C_t, mean_n_t, mean_s_t, is_weights,
                                 sum_det_weights);
  }

 private:
  sgdlm_handle h_ = nullptr;
};

}  // namespace

// The factory's three forms (HostWrapperFactory.cu:5-35), for the reference's
// build type DOUBLETYPE = double (rSGDLM/src/Makevars.in:1).
template <>
SGDLM::HostWrapper<double> *SGDLM::HostWrapperFactory<double>::create(std::size_t no_gpus) {
  return new GB300HostWrapper(no_gpus);
}

template <>
SGDLM::HostWrapper<double> *SGDLM::HostWrapperFactory<double>::create(std::size_t no_gpus,
                                                                     std::size_t m,
                                                                     std::size_t max_p) {
  SGDLM::HostWrapper<double> *w = new GB300HostWrapper(no_gpus);
  w->initMemory(m, max_p);
  return w;
}

template <>
SGDLM::HostWrapper<double> *SGDLM::HostWrapperFactory<double>::create(
    std::size_t no_gpus, std::size_t m, std::size_t max_p, bool use_evolution_matrix) {
  SGDLM::HostWrapper<double> *w = new GB300HostWrapper(no_gpus);
  w->initMemory(m, max_p);
  w->manageEvoMemory(use_evolution_matrix);
  return w;
}
