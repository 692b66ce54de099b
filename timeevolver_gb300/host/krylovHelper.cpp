// krylovHelper.cpp -- result output (helper/krylovHelper.cpp:10-203 of
// TimeEvolver): the CSV branch of saveResult, and its HDF5 branch plus
// saveMatrix / saveSparseMatrix through the library's own HDF5 writer.
#define USE_HDF
#include "krylovHelper.h"

#include <ctime>
#include <fstream>

#include "h5min.h"

namespace {

std::string result_base(parameter_list& para, const std::string& name) {
  std::string base = name;
  for (const std::shared_ptr<parameter>& p : para)
    if (p->getPrintFilename()) base += "_" + p->getName() + p->getData();
  return base;
}

uint32_t now() { return (uint32_t)std::time(nullptr); }

}  // namespace

void saveResultCSV(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                   const std::string& name) {
  const std::string base = result_base(para, name);
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

// One dataset per observable (its samples), every parameter attached as an
// attribute in list order: doubles as IEEE doubles, ints and bools as int32
// (helper/krylovHelper.cpp:34-89).
void saveResultHDF5(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                    const std::string& name) {
  std::vector<h5min::Attribute> attrs;
  for (const std::shared_ptr<parameter>& p : para) {
    h5min::Attribute a;
    a.name = p->getName();
    if (p->isDouble()) {
      a.is_double = true;
      a.d = dynamic_cast<typedParameter<double>&>(*p).getValue();
    } else if (p->isInt()) {
      a.is_double = false;
      a.i = dynamic_cast<typedParameter<int>&>(*p).getValue();
    } else if (p->isBool()) {
      a.is_double = false;
      a.i = dynamic_cast<typedParameter<bool>&>(*p).getValue() ? 1 : 0;
    } else {
      continue;  // other parameter types are not written (as in the reference)
    }
    attrs.push_back(a);
  }
  h5min::File f;
  for (const std::unique_ptr<krylovBasicObservable>& obs : obs_list)
    f.add(obs->retName(), obs->retExpectationValues(), obs->retNumSamples(), attrs);
  f.write(result_base(para, name) + ".h5", now());
}

void saveMatrix(const matrix* mat, const std::string& name) {
  std::vector<double> re(mat->numValues), im(mat->numValues);
  for (size_t i = 0; i < mat->numValues; ++i) {
    re[i] = mat->values[i].real();
    im[i] = mat->values[i].imag();
  }
  h5min::File f;
  f.add("valuesRealPart", re.data(), re.size());
  f.add("valuesImagPart", im.data(), im.size());
  f.write(name, now());
}

void saveSparseMatrix(const smatrix* mat, const std::string& name) {
  std::vector<double> re(mat->numValues), im(mat->numValues);
  for (size_t i = 0; i < mat->numValues; ++i) {
    re[i] = mat->values[i].real();
    im[i] = mat->values[i].imag();
  }
  std::vector<uint64_t> col(mat->columns, mat->columns + mat->numValues);
  std::vector<uint64_t> row(mat->rowIndex, mat->rowIndex + mat->numValues);
  const uint64_t dim = (uint64_t)mat->m;
  h5min::File f;
  f.add("valuesRealPart", re.data(), re.size());
  f.add("valuesImagPart", im.data(), im.size());
  f.add("columIndex", col.data(), col.size());
  f.add("rowIndex", row.data(), row.size());
  f.add("dimension", &dim, 1);
  f.write(name, now());
}
