// Force-included ahead of every reference translation unit (g++ -include).
// The reference targets MSVC: it relies on transitive standard includes and
// on _aligned_malloc/_aligned_free. This header supplies both on Linux.
// Test infrastructure only.
#pragma once
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <optional>
#include <random>
#include <stack>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
using std::isfinite;
using std::isnan;
inline void* _aligned_malloc(size_t size, size_t align) {
  size_t rounded = (size + align - 1) / align * align;
  return std::aligned_alloc(align, rounded ? rounded : align);
}
inline void _aligned_free(void* p) { std::free(p); }
