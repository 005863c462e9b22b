/* ISPC language support for C++ at gang size one (TEST INFRASTRUCTURE ONLY).
 *
 * oracle/ispc_ref.py translates the reference's *.ispc sources into C++ that
 * includes this header first.  At a gang size of one every "varying" value
 * has one program instance, so:
 *
 *   - uniform and varying qualifiers are empty; cif/cfor/cwhile are if/for/while;
 *   - reduce_add/min/max, any and all of one lane return that lane's value
 *     (sums of lane partials become sums in loop order);
 *   - a launch of n tasks runs task indices 0..n-1, in order when one thread is
 *     used and spread over OpenMP threads otherwise, and returns when all have
 *     run (so sync is empty);
 *   - the atomics are GCC atomic builtins; the store of -1 that releases a
 *     list lock is a release store (ispc_unlock), which is what the x86
 *     targets the reference is built for give a plain store;
 *   - new and delete map to calloc and free: blocks start zeroed, as the
 *     reference's aligned_real_alloc and master_alloc leave them.
 */
#ifndef ISPC_GANG1_H
#define ISPC_GANG1_H

#include <cassert>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

#define uniform
#define varying
#define cif if
#define cfor for
#define cwhile while
#define cdo do

typedef unsigned int uint;
typedef int8_t int8;
typedef uint8_t uint8;
typedef int16_t int16;
typedef uint16_t uint16;
typedef int32_t int32;
typedef uint32_t uint32;
typedef int64_t int64;
typedef uint64_t uint64;

using std::abs;
using std::sqrt;
using std::sin;
using std::cos;
using std::acos;
using std::floor;
using std::ceil;
using std::pow;
using std::exp;
using std::log;

template <class A, class B>
static inline typename std::common_type<A, B>::type min(A a, B b)
{
  typedef typename std::common_type<A, B>::type T;
  return (T)a < (T)b ? (T)a : (T)b;
}
template <class A, class B>
static inline typename std::common_type<A, B>::type max(A a, B b)
{
  typedef typename std::common_type<A, B>::type T;
  return (T)a > (T)b ? (T)a : (T)b;
}

template <class T> static inline T reduce_add(T x) { return x; }
template <class T> static inline T reduce_min(T x) { return x; }
template <class T> static inline T reduce_max(T x) { return x; }
static inline bool any(bool x) { return x; }
static inline bool all(bool x) { return x; }
template <class T> static inline T select(bool c, T a, T b) { return c ? a : b; }

template <class T> static inline T atomic_compare_exchange_global(T *p, T expected, T desired)
{
  return __sync_val_compare_and_swap(p, expected, desired);
}
template <class T, class V> static inline T atomic_add_global(T *p, V v) { return __sync_fetch_and_add(p, (T)v); }
template <class T, class V> static inline T atomic_min_global(T *p, V v)
{
  T old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while ((T)v < old && !__atomic_compare_exchange_n(p, &old, (T)v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return old;
}
template <class T, class V> static inline T atomic_max_global(T *p, V v)
{
  T old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while ((T)v > old && !__atomic_compare_exchange_n(p, &old, (T)v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
  return old;
}
template <class T> static inline void ispc_unlock(T *p) { __atomic_store_n(p, (T)-1, __ATOMIC_RELEASE); }

template <class T> static inline T *ispc_new(long n) { return (T *)calloc(n > 0 ? (size_t)n : 1, sizeof(T)); }
static inline void ispc_delete(void *p) { free(p); }

/* ISPC's print takes '%' for every argument; the translation keeps the
   reference's diagnostics as one line with the format only. */
static inline void ispc_print(const char *fmt, ...) { fputs(fmt, stderr); }

/* The reference's constants.h wraps its enums in namespace parmec when it is
   compiled as C++; ISPC sees them at global scope. */
namespace parmec {}
using namespace parmec;

static inline int num_cores()
{
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

/* task context of the running program instance */
static thread_local int taskIndex = 0;
static thread_local int taskCount = 1;

#define ISPC_SYNC ((void)0)

#ifdef _OPENMP
#define ISPC_LAUNCH(n, call)                                                                   \
  do {                                                                                         \
    const int ispc_n_ = (n);                                                                   \
    const int ispc_ti_ = taskIndex, ispc_tc_ = taskCount;                                      \
    if (ispc_n_ <= 1 || omp_in_parallel()) {                                                   \
      for (int ispc_t_ = 0; ispc_t_ < ispc_n_; ispc_t_++) {                                    \
        taskIndex = ispc_t_; taskCount = ispc_n_; call;                                        \
      }                                                                                        \
    } else {                                                                                   \
      _Pragma("omp parallel for schedule(dynamic, 1)")                                         \
      for (int ispc_t_ = 0; ispc_t_ < ispc_n_; ispc_t_++) {                                    \
        taskIndex = ispc_t_; taskCount = ispc_n_; call;                                        \
      }                                                                                        \
    }                                                                                          \
    taskIndex = ispc_ti_; taskCount = ispc_tc_;                                                \
  } while (0)
#else
#define ISPC_LAUNCH(n, call)                                                                   \
  do {                                                                                         \
    const int ispc_n_ = (n);                                                                   \
    const int ispc_ti_ = taskIndex, ispc_tc_ = taskCount;                                      \
    for (int ispc_t_ = 0; ispc_t_ < ispc_n_; ispc_t_++) {                                      \
      taskIndex = ispc_t_; taskCount = ispc_n_; call;                                          \
    }                                                                                          \
    taskIndex = ispc_ti_; taskCount = ispc_tc_;                                                \
  } while (0)
#endif

#endif
