/*
 * CPU restatement of libcint 6.1.1's Rys-quadrature two-electron integrals (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load
 * this library, and only as the thing the CUDA path is checked against (or as the timed CPU
 * port).  The product library (libcintgpu.so) never links or calls it.
 *
 * Entry points take libcint's exact argument lists (libcint include/cint_funcs.h:11-15) so a
 * test can run the reference library, this restatement and the CUDA drop-in on identical
 * atm/bas/env and compare element by element.
 *
 * Roots and weights are computed by an algorithm independent of both libcint's polynomial fits
 * and the GPU tables: a discretised Stieltjes procedure on a Gauss-Legendre rule followed by a
 * Golub-Welsch eigen-decomposition of the Jacobi matrix.
 */
#ifndef ORACLE_RYS_H
#define ORACLE_RYS_H
#ifdef __cplusplus
extern "C" {
#endif

/* u[i] = t_i^2/(1-t_i^2), w[i] = weights of int_0^1 f(t^2) exp(-x t^2) dt; mirrors
 * CINTrys_roots (libcint src/rys_roots.c:57-122). Returns 0 on success. */
int oracle_rys_roots(int nroots, double x, double *u, double *w);
/* the same for the weight restricted to t in [lower, 1] (short-range Coulomb: lower = sqrt(theta)) */
int oracle_rys_roots_range(int nroots, double x, double lower, double *u, double *w);

/* Same meaning and argument order as libcint's int2e_sph etc. opt and cache are ignored
 * (the restatement always takes the no-optimizer path, src/cint2e.c:57-269). */
int oracle_int2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                     int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                      int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2e_ip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                         int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2e_ip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                          int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                       int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                        int *bas, int nbas, double *env, void *opt, double *cache);
/* (ij|nabla k l), (nabla i j|k), (ij|nabla k): libcint src/autocode/grad2.c:163-176,
 * src/autocode/int3c2e.c:72-87, :153-168 */
int oracle_int2e_ip2_sph(double *out, int *dims, int *shls, int *atm, int natm,
                         int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2e_ip2_cart(double *out, int *dims, int *shls, int *atm, int natm,
                          int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_ip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_ip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_ip2_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int3c2e_ip2_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache);
/* (nabla nabla i j|kl), 9 components 3p + q (libcint src/autocode/hess.c:1124-1194) */
int oracle_int2e_ipip1_sph(double *out, int *dims, int *shls, int *atm, int natm,
                           int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2e_ipip1_cart(double *out, int *dims, int *shls, int *atm, int natm,
                            int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2c2e_sph(double *out, int *dims, int *shls, int *atm, int natm,
                       int *bas, int nbas, double *env, void *opt, double *cache);
int oracle_int2c2e_cart(double *out, int *dims, int *shls, int *atm, int natm,
                        int *bas, int nbas, double *env, void *opt, double *cache);

/* Cartesian -> real solid harmonic coefficient matrix for angular momentum l, written as
 * c[m*ncart + icart] (2l+1 rows).  l = 0,1 give the identity (their factors live in the
 * common factor, libcint src/g1e.c:565-572).  Returns the number of rows. */
int oracle_cart2sph_coeff(int l, double *c);

/* Evaluate a list of shell quartets (4 ints each) through oracle_int2e_sph with OpenMP
 * over quartets (the harness pattern of libcint examples/time_c2h6.c:719-745).  Each quartet
 * writes its dense block at out + offsets[q]; out may be NULL to only time.  Returns wall
 * seconds.  nthreads <= 0 uses the OpenMP default. */
double oracle_int2e_sph_list(const int *quartets, long nq, double *out, const long *offsets,
                             int *atm, int natm, int *bas, int nbas, double *env, int nthreads);

/* Any kind over a list of items (which: 0 int2e_sph, 1 int2e_cart, 2 int2e_ip1_sph,
 * 3 int2e_ip1_cart, 4 int3c2e_sph, 5 int3c2e_cart, 6 int2c2e_sph, 7 int2c2e_cart, 8 int2e_ip2_sph,
 * 9 int2e_ip2_cart, 10 int3c2e_ip1_sph, 11 int3c2e_ip1_cart, 12 int3c2e_ip2_sph,
 * 13 int3c2e_ip2_cart, 14 int2e_ipip1_sph, 15 int2e_ipip1_cart), OpenMP over
 * items, dense blocks (all components) at out + offsets[q].  Returns wall seconds. */
double oracle_list(int which, const int *items, long n, double *out, const long *offsets,
                   int *atm, int natm, int *bas, int nbas, double *env, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
