/*
 * CPU timing harness for a shell-quartet list -- TEST / BASELINE INFRASTRUCTURE.
 *
 * Follows the pattern of libcint examples/time_c2h6.c:686-760: one optimizer, then OpenMP
 * schedule(dynamic) over the quartets, wall time from omp_get_wtime.  Linked against libcint
 * itself (oracle/_ref/ref_bench) or, with -DUSE_ORACLE, against the C restatement
 * (oracle/_build/oracle_bench) so both are timed by identical code.
 *
 * usage: ref_bench <input.bin> <nthreads> [repeat]
 * input.bin: int32 natm, nbas, nenv, nq; int32 atm[natm*6]; int32 bas[nbas*8];
 *            float64 env[nenv]; int32 quartets[nq*4]
 * prints one JSON line: seconds, threads, quartets, integrals (sph), checksum sum|v|.
 */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <omp.h>

#ifdef USE_ORACLE
#include "oracle_rys.h"
#define INT2E_SPH(out, dims, shls, atm, natm, bas, nbas, env, opt, cache) \
        oracle_int2e_sph(out, dims, shls, atm, natm, bas, nbas, env, opt, cache)
typedef void CINTOpt;
static void make_opt(CINTOpt **opt, int *atm, int natm, int *bas, int nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)nbas; (void)env; *opt = NULL; }
static void free_opt(CINTOpt **opt) { *opt = NULL; }
#define IMPL "port"
#else
#include "cint.h"
int int2e_sph(double *out, int *dims, int *shls, int *atm, int natm, int *bas, int nbas,
              double *env, CINTOpt *opt, double *cache);
void int2e_optimizer(CINTOpt **opt, int *atm, int natm, int *bas, int nbas, double *env);
#define INT2E_SPH int2e_sph
static void make_opt(CINTOpt **opt, int *atm, int natm, int *bas, int nbas, double *env)
{ int2e_optimizer(opt, atm, natm, bas, nbas, env); }
static void free_opt(CINTOpt **opt) { CINTdel_optimizer(opt); }
#define IMPL "reference"
#endif

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: %s input.bin nthreads [repeat]\n", argv[0]); return 2; }
    FILE *f = fopen(argv[1], "rb");
    if (!f) { perror(argv[1]); return 2; }
    int hdr[4];
    if (fread(hdr, sizeof(int), 4, f) != 4) return 2;
    int natm = hdr[0], nbas = hdr[1], nenv = hdr[2], nq = hdr[3];
    int *atm = malloc(sizeof(int) * natm * 6);
    int *bas = malloc(sizeof(int) * nbas * 8);
    double *env = malloc(sizeof(double) * nenv);
    int *q = malloc(sizeof(int) * (size_t)nq * 4);
    if (fread(atm, sizeof(int), natm * 6, f) != (size_t)natm * 6) return 2;
    if (fread(bas, sizeof(int), nbas * 8, f) != (size_t)nbas * 8) return 2;
    if (fread(env, sizeof(double), nenv, f) != (size_t)nenv) return 2;
    if (fread(q, sizeof(int), (size_t)nq * 4, f) != (size_t)nq * 4) return 2;
    fclose(f);
    int nthreads = atoi(argv[2]);
    int repeat = argc > 3 ? atoi(argv[3]) : 1;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    int used = 1;
#pragma omp parallel
    {
#pragma omp master
        used = omp_get_num_threads();
    }
    CINTOpt *opt = NULL;
    make_opt(&opt, atm, natm, bas, nbas, env);
    double nint = 0;
    for (long i = 0; i < nq; i++) {
        double n = 1;
        for (int a = 0; a < 4; a++) {
            int *b = bas + 8 * q[4 * i + a];
            n *= (2 * b[1] + 1) * b[3];
        }
        nint += n;
    }
    double checksum = 0, t0 = omp_get_wtime();
    for (int rep = 0; rep < repeat; rep++) {
        checksum = 0;
#pragma omp parallel reduction(+:checksum)
        {
            double *buf = malloc(sizeof(double) * 160000);
#pragma omp for schedule(dynamic, 2)
            for (long i = 0; i < nq; i++) {
                int *s = q + 4 * i;
                int n = 1;
                for (int a = 0; a < 4; a++) {
                    int *b = bas + 8 * s[a];
                    n *= (2 * b[1] + 1) * b[3];
                }
                INT2E_SPH(buf, NULL, s, atm, natm, bas, nbas, env, opt, NULL);
                for (int k = 0; k < n; k++) checksum += fabs(buf[k]);
            }
            free(buf);
        }
    }
    double t1 = omp_get_wtime();
    free_opt(&opt);
    printf("{\"impl\": \"%s\", \"seconds\": %.6f, \"threads\": %d, \"quartets\": %d, "
           "\"integrals\": %.0f, \"repeat\": %d, \"checksum\": %.12e}\n",
           IMPL, (t1 - t0) / repeat, used, nq, nint, repeat, checksum);
    return 0;
}
