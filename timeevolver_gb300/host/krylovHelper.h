// krylovHelper.h -- saving sampled expectation values (same API as
// helper/krylovHelper.h of TimeEvolver).  The reference writes HDF5 when
// built with it and CSV otherwise; HDF5 is not part of this build, so
// saveResult takes the CSV branch: one file per observable,
//   <name>[_<param><value> for every parameter flagged for the file name]<observable name>.csv
// holding the samples separated by ", " in the default stream format.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "krylovObservables.h"
#include "parameter.h"

void saveResult(const std::vector<std::unique_ptr<krylovBasicObservable>>& obs_list, parameter_list& para,
                const std::string& name);
