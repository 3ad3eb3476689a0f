/* voss_numbers.h -- the arithmetic-functions part of the voss C ABI.
 *
 * Same declarations as the reference's library/include/voss/voss_numbers.h
 * (lines 16-45).  These functions are not part of the sieve; the library
 * exports them only so that the reference's ctypes binding, which binds every
 * symbol at import (bindings/python/voss/_capi.py:263-312), loads.  Each one
 * returns VOSS_ERR_INTERNAL with a message.
 */
#ifndef VOSS_NUMBERS_H
#define VOSS_NUMBERS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int voss_numbers_phi(uint64_t n, uint64_t* out);
int voss_numbers_tau(uint64_t n, uint64_t* out);
int voss_numbers_sigma(uint64_t n, uint64_t* out);
int voss_numbers_mu(uint64_t n, int* out);
int voss_numbers_gcd(uint64_t a, uint64_t b, uint64_t* out);
int voss_numbers_lcm(uint64_t a, uint64_t b, uint64_t* out);
int voss_numbers_fibonacci(uint64_t n, uint64_t* out);
int voss_numbers_factorial(uint64_t n, uint64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* VOSS_NUMBERS_H */
