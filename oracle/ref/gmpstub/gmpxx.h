/*
 * Declaration-only stand-in for <gmpxx.h>, used ONLY to compile the reference
 * sources (prothlogic4.2/proth_logic.cpp, storage_core.cpp) into the test
 * harness under oracle/_ref.  It declares the handful of public GMP C functions
 * those files call, with GMP's documented signatures and its documented mpz_t
 * layout, and links against the system's libgmp.so.10.  No GMP code is here.
 */
#ifndef PROTH_GMP_DECL_STUB_H
#define PROTH_GMP_DECL_STUB_H
#include <cstddef>
extern "C" {
typedef unsigned long mp_limb_t;
typedef struct { int _mp_alloc; int _mp_size; mp_limb_t* _mp_d; } __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;
void __gmpz_init(mpz_ptr);
void __gmpz_inits(mpz_ptr, ...);
void __gmpz_clear(mpz_ptr);
void __gmpz_set_ui(mpz_ptr, unsigned long);
void __gmpz_mul_2exp(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_sub_ui(mpz_ptr, mpz_srcptr, unsigned long);
int __gmpz_jacobi(mpz_srcptr, mpz_srcptr);
void __gmpz_powm(mpz_ptr, mpz_srcptr, mpz_srcptr, mpz_srcptr);
void* __gmpz_export(void*, size_t*, int, size_t, int, size_t, mpz_srcptr);
void __gmpz_import(mpz_ptr, size_t, int, size_t, int, size_t, const void*);
void __gmpz_mod(mpz_ptr, mpz_srcptr, mpz_srcptr);
char* __gmpz_get_str(char*, int, mpz_srcptr);
int __gmpz_cmp(mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
}
#define mpz_init __gmpz_init
#define mpz_inits __gmpz_inits
#define mpz_clear __gmpz_clear
#define mpz_set_ui __gmpz_set_ui
#define mpz_mul_2exp __gmpz_mul_2exp
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_add_ui __gmpz_add_ui
#define mpz_sub_ui __gmpz_sub_ui
#define mpz_jacobi __gmpz_jacobi
#define mpz_powm __gmpz_powm
#define mpz_export __gmpz_export
#define mpz_import __gmpz_import
#define mpz_mod __gmpz_mod
#define mpz_get_str __gmpz_get_str
#define mpz_cmp __gmpz_cmp
#define mpz_mul __gmpz_mul
/* opaque placeholder: the C++ wrapper type is named in a header but unused on this path */
class mpz_class { __mpz_struct placeholder_; };
#endif
