// krylovHelper.h -- saving sampled expectation values and matrices (same API
// as helper/krylovHelper.h of TimeEvolver).  As in the reference, the format
// of saveResult is chosen when the caller compiles: with USE_HDF it writes
// one HDF5 file
//   <name>[_<param><value> for every parameter flagged for the file name].h5
// holding a float64 dataset per observable with every parameter as a
// one-element attribute (double, or int32 for int and bool parameters), and
// saveMatrix / saveSparseMatrix are declared; without it, one CSV file per
// observable
//   <name>[_<param><value> ...]<observable name>.csv
// holding the samples separated by ", " in the default stream format.  The
// HDF5 files come from this library's own writer (h5min.h); no HDF5 library
// is needed, and none of its API is exported.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "krylovObservables.h"
#include "parameter.h"

// The two branches of saveResult (helper/krylovHelper.cpp:27-92 and :93-108).
void saveResultHDF5(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                    const std::string& name);
void saveResultCSV(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                   const std::string& name);

inline void saveResult(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                       const std::string& name) {
#ifdef USE_HDF
  saveResultHDF5(obs_list, para, name);
#else
  saveResultCSV(obs_list, para, name);
#endif
}

#ifdef USE_HDF
// Dense matrix: datasets valuesRealPart, valuesImagPart (helper/krylovHelper.cpp:160-203).
void saveMatrix(const matrix* mat, const std::string& name);
// Sparse matrix: valuesRealPart, valuesImagPart, columIndex, rowIndex (uint64)
// and the one-element dimension (helper/krylovHelper.cpp:112-155).
void saveSparseMatrix(const smatrix* mat, const std::string& name);
#endif
