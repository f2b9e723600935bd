// Prints the pointer-to-member representation of every virtual function of
// SGDLM::HostWrapper<double> (tests/test_host_wrapper.py).  Under the Itanium
// C++ ABI that representation encodes the function's vtable slot, so two builds
// -- one against include/sgdlm_hostwrapper.hpp, one against the reference's
// rSGDLM/src/SGDLM/HostWrapper.hpp (-DSGDLM_USE_REFERENCE_HEADERS) -- print the
// same lines exactly when a caller compiled against either header reaches the
// same implementation.
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>

#ifdef SGDLM_USE_REFERENCE_HEADERS
#include "SGDLM/HostWrapper.hpp"
#else
#include "sgdlm_hostwrapper.hpp"
#endif

using HW = SGDLM::HostWrapper<double>;

template <typename F> void show(const char *name, F f) {
  unsigned char raw[sizeof(F)];
  std::memcpy(raw, &f, sizeof(F));
  std::printf("%s", name);
  for (std::size_t i = 0; i < sizeof(F); ++i) std::printf(" %02x", raw[i]);
  std::printf("\n");
}

int main() {
  show("getNoSeries", &HW::getNoSeries);
  show("getMaxP", &HW::getMaxP);
  show("getEvolutionMatrixConfiguration", &HW::getEvolutionMatrixConfiguration);
  show("initMemory", &HW::initMemory);
  show("clearMemory", &HW::clearMemory);
  show("manageEvoMemory", &HW::manageEvoMemory);
  show("getNSim", &HW::getNSim);
  show("getNSimBatch", &HW::getNSimBatch);
  show("initSimMemory", &HW::initSimMemory);
  show("clearSimMemory", &HW::clearSimMemory);
  show("initForecastPriors", &HW::initForecastPriors);
  show("isPrior()", static_cast<bool (HW::*)() const>(&HW::isPrior));
  show("isPrior(bool)", static_cast<void (HW::*)(bool)>(&HW::isPrior));
  show("getParameters", &HW::getParameters);
  show("setParameters", &HW::setParameters);
  show("getDiscountFactors", &HW::getDiscountFactors);
  show("setDiscountFactors", &HW::setDiscountFactors);
  show("getEvolutionMatrix", &HW::getEvolutionMatrix);
  show("setEvolutionMatrix", &HW::setEvolutionMatrix);
  show("getParentalSets", &HW::getParentalSets);
  show("setParentalSets", &HW::setParentalSets);
  show("computePrior(bool)", static_cast<void (HW::*)(bool)>(&HW::computePrior));
  show("computePrior(G, bool)",
       static_cast<void (HW::*)(const double *, bool)>(&HW::computePrior));
  show("evolveForecastSamples()", static_cast<void (HW::*)()>(&HW::evolveForecastSamples));
  show("evolveForecastSamples(G)",
       static_cast<void (HW::*)(const double *)>(&HW::evolveForecastSamples));
  show("computeForecast", &HW::computeForecast);
  show("computePosterior", &HW::computePosterior);
  show("computeVBPosterior", &HW::computeVBPosterior);
  return 0;
}
