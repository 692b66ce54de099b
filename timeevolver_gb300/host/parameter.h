// parameter.h -- model parameters attached to saved results (same API as
// helper/parameter.h of TimeEvolver: parameter, typedParameter<T>,
// parameter_list, paraPush).  A parameter has a name, a value and a flag that
// puts "_<name><value>" into the output file name; the value is rendered with
// 10 significant digits, as the reference does, so file names agree.
#pragma once

#include <iomanip>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

class parameter {
 public:
  parameter(const std::string& name, bool inclInFilename) : p_name(name), includeInFilename(inclInFilename) {}
  parameter() = default;
  virtual ~parameter() {}
  virtual std::string getData() = 0;
  virtual bool isDouble() = 0;
  virtual bool isInt() = 0;
  virtual bool isBool() = 0;
  std::string getName() { return p_name; }
  bool getPrintFilename() { return includeInFilename; }

 private:
  std::string p_name;
  bool includeInFilename = false;
};

template <typename T>
class typedParameter : public parameter {
 public:
  typedParameter(const std::string& name, bool inclInFilname, const T& data)
      : parameter(name, inclInFilname), para_data(data) {}

  std::string getData() {
    std::ostringstream text;
    text << std::setprecision(10) << para_data;
    return text.str();
  }
  bool isDouble() { return std::is_same<T, double>::value; }
  bool isInt() { return std::is_same<T, int>::value; }
  bool isBool() { return std::is_same<T, bool>::value; }
  T getValue() { return para_data; }

 private:
  T para_data;
};

typedef std::vector<std::shared_ptr<parameter>> parameter_list;

// paraPush("name", inFilename, value): a shared typedParameter of the value's type.
#define paraPush(nm, bfnm, ...) std::make_shared<typedParameter<decltype(__VA_ARGS__)>>(nm, bfnm, __VA_ARGS__)
