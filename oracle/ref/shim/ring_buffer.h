// Stand-in for the pci-ring-buffer C header (test infrastructure for the reference pin).
// The hot path with ATOMICS tile distribution moves no data through ring buffers;
// only the type names, request macros and the atomics below are needed.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#ifndef likely
#define likely(x) __builtin_expect(!!(x), 1)
#define unlikely(x) __builtin_expect(!!(x), 0)
#endif
#define L1D_CACHELINE_SIZE 64

struct ring_buffer_t {
  int unused;
};
struct ring_buffer_req_t {
  size_t size;
  void* data;
  int rc;
  int flag;
};
typedef void (*ring_buffer_reap_cb_t)(void*, void*);

#define ring_buffer_get_req_init(req, md) \
  do {                                    \
    (req)->size = 0;                      \
    (req)->data = 0;                      \
    (req)->rc = 0;                        \
    (req)->flag = 0;                      \
  } while (0)
#define ring_buffer_put_req_init(req, md, sz) \
  do {                                        \
    ring_buffer_get_req_init(req, md);        \
    (req)->size = (sz);                       \
  } while (0)

// Sequentially consistent atomics with the semantics the reference expects.
template <class T, class U, class V>
static inline bool smp_cas(T* p, U expected, V desired) {
  T e = static_cast<T>(expected);
  return __atomic_compare_exchange_n(p, &e, static_cast<T>(desired), false, __ATOMIC_SEQ_CST,
                                     __ATOMIC_SEQ_CST);
}
// 32-bit CAS on the first word of *p, comparing the bit patterns of the values.
template <class P, class V>
static inline bool smp_cas_float(P* p, const V& expected, const V& desired) {
  uint32_t e, d;
  memcpy(&e, &expected, 4);
  memcpy(&d, &desired, 4);
  return __atomic_compare_exchange_n(reinterpret_cast<uint32_t*>(p), &e, d, false, __ATOMIC_SEQ_CST,
                                     __ATOMIC_SEQ_CST);
}
template <class T, class U>
static inline T smp_faa(T* p, U v) {
  return __atomic_fetch_add(p, static_cast<T>(v), __ATOMIC_SEQ_CST);
}
