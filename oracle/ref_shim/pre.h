// Force-included before the reference's src/cochlea.cu when it is compiled to
// a cubin.  The reference targets MSVC: its header declares functions with
// the dynamic exception specification `throw(...)` and its host code calls
// memcpy_s.  The standard headers are included first (so the macro below
// cannot reach them), then `throw(...)` is defined away and memcpy_s given a
// plain definition.  Neither touches device code.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <iterator>
#include <locale>
#include <map>
#include <memory>
#include <mutex>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>
#define throw(...)
inline int memcpy_s(void* d, size_t n, const void* s, size_t c) {
  (void)n;
  std::memcpy(d, s, c);
  return 0;
}
