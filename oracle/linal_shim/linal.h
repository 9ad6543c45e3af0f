/*
 * Minimal stand-in for the un-vendored "linal" headers, written for this
 * project so that the reference's own sources (src/, examples/, utils/)
 * compile into oracle/_ref.  TEST INFRASTRUCTURE ONLY.
 *
 * Semantics follow the reference call sites (examples/barvortex_impl.h:237-272
 * comments): vec_sum r=a+b, vec_sum1 r=k1*a+k2*b, vec_sum2 r=a+k*b,
 * vec_diff r=a-b, vec_mult r=a*b, vec_mult_scalar r=k*a, vec_scalar2 = dot.
 */
#ifndef ORC_LINAL_SHIM_H
#define ORC_LINAL_SHIM_H
#include <vector>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cassert>
#include <cstdlib>
#include "pow.h"
#include "timer.h"

namespace linal {

template <typename T> struct Allocator {};

template <typename T, typename Alloc = Allocator<T> >
class Array : public std::vector<T> {
public:
	Array() {}
	explicit Array(size_t n) : std::vector<T>(n) {}
};

template <typename T> class ArrayHost : public Array<T> {
public:
	ArrayHost() {}
	explicit ArrayHost(size_t n) : Array<T>(n) {}
};

template <typename T> class ArrayDevice : public Array<T> {
public:
	ArrayDevice() {}
	explicit ArrayDevice(size_t n) : Array<T>(n) {}
};

template <typename T, typename A, typename B>
void vec_sum(T *r, const A *a, const B *b, int n) { for (int i = 0; i < n; ++i) r[i] = a[i] + b[i]; }
template <typename T, typename A, typename B, typename K>
void vec_sum1(T *r, const A *a, const B *b, K k1, K k2, int n) { for (int i = 0; i < n; ++i) r[i] = k1 * a[i] + k2 * b[i]; }
template <typename T, typename A, typename B, typename K>
void vec_sum2(T *r, const A *a, const B *b, K k, int n) { for (int i = 0; i < n; ++i) r[i] = a[i] + k * b[i]; }
template <typename T>
void vec_diff(T *r, const T *a, const T *b, int n) { for (int i = 0; i < n; ++i) r[i] = a[i] - b[i]; }
template <typename T>
void vec_mult(T *r, const T *a, const T *b, int n) { for (int i = 0; i < n; ++i) r[i] = a[i] * b[i]; }
template <typename T, typename K>
void vec_mult_scalar(T *r, const T *a, K k, int n) { for (int i = 0; i < n; ++i) r[i] = k * a[i]; }
template <typename T>
T vec_scalar2(const T *a, const T *b, int n) { T s = 0; for (int i = 0; i < n; ++i) s += a[i] * b[i]; return s; }
template <typename T>
void vec_copy_from_host(T *d, const T *s, int n) { memcpy(d, s, sizeof(T) * n); }
template <typename T>
void vec_copy_from_device(T *d, const T *s, int n) { memcpy(d, s, sizeof(T) * n); }
template <typename T>
void vec_print(FILE *f, const T *a, int n, const char *fmt) { for (int i = 0; i < n; ++i) fprintf(f, fmt, (double)a[i]); fprintf(f, "\n"); }

inline void linal_init() {}
inline void linal_shutdown() {}
inline void set_num_threads(int) {}
inline bool check_device_supports_double() { return true; }

} /* namespace linal */
#endif
