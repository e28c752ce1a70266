/*
 * gmp.h -- declaration shim for compiling the reference's CPU path
 * (cuda/helper.h) against the installed GMP 6 runtime (libgmp.so.10), whose
 * development headers are not installed.  It declares only the public mpz
 * ABI that helper.h uses: the __mpz_struct layout, the __gmpz_* / __gmp_*
 * entry points and the mpz_* / gmp_* names GMP maps onto them.
 * Test infrastructure for the oracle; the library never includes it.
 */
#ifndef ORACLE_REF_GMP_SHIM_H
#define ORACLE_REF_GMP_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
    int _mp_alloc;
    int _mp_size;
    void* _mp_d;
} __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;
typedef struct {
    mpz_t _mp_seed;
    int _mp_alg;
    void* _mp_algdata;
} __gmp_randstate_struct;
typedef __gmp_randstate_struct gmp_randstate_t[1];

void __gmpz_init(mpz_ptr);
void __gmpz_clear(mpz_ptr);
void __gmpz_import(mpz_ptr, size_t, int, size_t, int, size_t, const void*);
void* __gmpz_export(void*, size_t*, int, size_t, int, size_t, mpz_srcptr);
void __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_rrandomb(mpz_ptr, __gmp_randstate_struct*, unsigned long);
int __gmp_printf(const char*, ...);
#ifdef __cplusplus
}
#endif
#define mpz_init __gmpz_init
#define mpz_clear __gmpz_clear
#define mpz_import __gmpz_import
#define mpz_export __gmpz_export
#define mpz_add __gmpz_add
#define mpz_mul __gmpz_mul
#define mpz_rrandomb __gmpz_rrandomb
#define gmp_printf __gmp_printf
#endif
