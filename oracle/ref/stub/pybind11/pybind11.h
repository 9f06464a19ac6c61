// Minimal stand-in for the one pybind11 facility the reference's PYBIND-mode
// InputData uses (pybind11::print).  Lets the reference's CUDA path be compiled
// and driven from a plain C++ harness on machines without Python headers.
// Test infrastructure only: it is part of the oracle, never of the product.
#pragma once
#include <algorithm>
#include <array>
#include <iostream>
#include <string>
#include <utility>
#include <vector>

namespace pybind11 {
template <class T>
inline std::ostream &operator<<(std::ostream &os, const std::vector<T> &v) {
  os << '[';
  for (size_t i = 0; i < v.size(); ++i) os << (i ? ", " : "") << v[i];
  return os << ']';
}
inline void print_one_(std::ostream &) {}
template <class T, class... Rest>
inline void print_one_(std::ostream &os, T &&v, Rest &&...rest) {
  os << v;
  if (sizeof...(rest)) os << ' ';
  print_one_(os, std::forward<Rest>(rest)...);
}
template <class... Args>
inline void print(Args &&...args) {
  print_one_(std::cout, std::forward<Args>(args)...);
  std::cout << '\n';
}
}  // namespace pybind11
