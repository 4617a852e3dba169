// iqs_gb300/utils.hpp -- the small helpers of intel/intel-qs's include/utils.hpp,
// include/conversion.hpp and include/bitops.hpp that callers of the register use: the UL()
// cast, iqs::toString, wall-clock seconds, and integer bit utilities.
#pragma once

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <sstream>
#include <stdexcept>
#include <string>

// Macros callers of the reference use (include/utils.hpp:6-20): compile-time notes, the
// size_t cast, seconds, stringification.
#ifndef DO_PRAGMA
#define DO_PRAGMA(x) _Pragma(#x)
#endif
#ifndef TODO
#define TODO(x) DO_PRAGMA(message("TODO - " #x))
#endif
#ifndef INFO
#define INFO(x) DO_PRAGMA(message("INFO - " #x))
#endif
#ifndef UL
#define UL(x) ((std::size_t)(x))
#endif
#ifndef sec
#define sec() iqs::time_in_seconds()
#endif
#ifndef __str__
#define __str__(s) #s
#endif
#ifndef xstr
#define xstr(s) __str__(s)
#endif

namespace iqs {

template <class T>
std::string toString(T const& val) {
  std::ostringstream os;
  os << val;
  return os.str();
}

inline double time_in_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Largest power of two not above x (1 for x = 0 or 1).
template <class Integral>
unsigned floor_power_of_two(Integral x) {
  unsigned p = 1;
  while (x >>= 1) p <<= 1;
  return p;
}

// Index of the highest set bit of a non-zero integer.
template <class Integral>
constexpr unsigned highestBit(Integral i) {
  unsigned pos = 0;
  while (i >>= 1) ++pos;
  return pos;
}

template <class Integral>
constexpr bool isPowerOf2(Integral i) {
  return i != static_cast<Integral>(0) && (i & (i - 1)) == 0;
}

// log2 of a power of two; throws std::invalid_argument otherwise (the reference asserts).
template <class Integral>
unsigned ilog2(Integral n) {
  if (!isPowerOf2(n)) throw std::invalid_argument("ilog2: not a power of 2");
  return highestBit(n);
}

inline long popcnt(uint32_t x) { return (long)__builtin_popcount(x); }
inline long popcnt(uint64_t x) { return (long)__builtin_popcountll(x); }

}  // namespace iqs
