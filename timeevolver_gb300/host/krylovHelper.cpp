// krylovHelper.cpp -- CSV output of sampled expectation values
// (helper/krylovHelper.cpp:10-110 of TimeEvolver, its non-HDF5 branch).
#include "krylovHelper.h"

#include <fstream>

void saveResult(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                const std::string& name) {
  std::string base = name;
  for (const std::shared_ptr<parameter>& p : para)
    if (p->getPrintFilename()) base += "_" + p->getName() + p->getData();
  for (const std::unique_ptr<krylovBasicObservable>& obs : obs_list) {
    std::ofstream out(base + obs->retName() + ".csv");
    const double* values = obs->retExpectationValues();
    const size_t count = obs->retNumSamples();
    for (size_t i = 0; i < count; ++i) {
      if (i > 0) out << ", ";
      out << values[i];
    }
  }
}
