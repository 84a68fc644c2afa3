// Force-included (-include) into the reference sources when building the
// oracle harness binary only.  The reference locates a face by a linear scan
// of the all-faces vector (cppnabla/utils/Utils.h:65-72); that vector is the
// identity 0..nbFaces-1 (cppnabla/mesh/CartesianMesh2D.cc:42-43), so the
// value is its own index.  This explicit specialisation returns that index in
// O(1) when vector[value] == value and otherwise falls back to the same scan,
// so every call returns exactly what the reference returns.  It only makes the
// harness usable on meshes beyond ~64x64 (the scan makes each cycle O(N^2)).
//
// It also opens class access (`private` -> `public`) for the rest of each
// translation unit so the harness can call the schemes' set-up steps one by
// one and read their state.  Every standard header the reference uses is
// included first, so the macro never reaches the standard library.
#ifndef ORACLE_REF_FASTPATH_H
#define ORACLE_REF_FASTPATH_H
#include <algorithm>
#include <array>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <exception>
#include <experimental/filesystem>
#include <fstream>
#include <functional>
#include <future>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>
#include <math.h>
#include <stdlib.h>
#include <stddef.h>

#include "utils/Utils.h"

namespace nablalib {
namespace utils {
template <>
inline size_t indexOf<size_t>(const std::vector<size_t>& vector,
                              const size_t& value) {
  if (value < vector.size() && vector[value] == value) return value;
  for (size_t i(0); i < vector.size(); ++i)
    if (vector[i] == value) return i;
  throw std::out_of_range("Value not in vector");
}
}  // namespace utils
}  // namespace nablalib

#define private public
#endif
