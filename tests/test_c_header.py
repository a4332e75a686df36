"""The drop-in from C: a C99 program that includes include/cintgpu.h exactly as a libcint caller
includes cint.h, links libcintgpu.so and calls the entries that need no GPU (basis helpers, the
out == NULL cache-size queries, an argument error and its message), compared with the values the
Python tests check; CPU only."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SRC = r"""
#include <stdio.h>
#include <math.h>
#include "cintgpu.h"

int main(int argc, char **argv)
{
    /* one s and one d shell on one atom: libcint's atm / bas / env layout */
    int atm[6] = {1, 20, 0, 0, 0, 0};
    int bas[16] = {0, 0, 2, 1, 0, 23, 25, 0,
                   0, 2, 1, 2, 0, 27, 28, 0};
    double env[40] = {0};
    env[23] = 1.3; env[24] = 0.4;
    env[25] = CINTgto_norm(0, 1.3); env[26] = CINTgto_norm(0, 0.4);
    env[27] = 0.8; env[28] = CINTgto_norm(2, 0.8); env[29] = 0.5 * CINTgto_norm(2, 0.8);
    printf("norm %.17g\n", CINTgto_norm(2, 0.8));
    printf("sph %d %d cart %d tot %d\n", CINTcgto_spheric(0, bas), CINTcgto_spheric(1, bas),
           CINTcgto_cart(1, bas), CINTtot_cgto_spheric(bas, 2));
    int shls[4] = {1, 0, 1, 1};
    printf("cache2e %d\n", (int)int2e_sph(NULL, NULL, shls, atm, 1, bas, 2, env, NULL, NULL));
    int sh2[2] = {1, 0};
    printf("cache2c %d\n", (int)int2c2e_sph(NULL, NULL, sh2, atm, 1, bas, 2, env, NULL, NULL));
    CINTOpt *opt = NULL;
    int2e_optimizer(&opt, atm, 1, bas, 2, env);
    printf("opt %d\n", opt != NULL);
    CINTdel_optimizer(&opt);
    printf("deleted %d\n", opt == NULL);
    CINTGPUPlan *plan = NULL;
    int bad[4] = {0, 0, 0, 9};
    int rc = cintgpu_plan_create_tuned(&plan, CINTGPU_INT2E_SPH, bad, 1, NULL, atm, 1, bas, 2, env,
                                       4, 0);
    printf("rc %d msg %s\n", rc, cintgpu_last_error());
    return 0;
}
"""


def test_c_program_against_the_header(gpulib, tmp_path):
    import shutil
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    lib = gpulib.lib()._name
    src = tmp_path / 'caller.c'
    src.write_text(C_SRC)
    exe = tmp_path / 'caller'
    subprocess.run([cc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'),
                    str(src), lib, '-lm', '-o', str(exe),
                    '-Wl,-rpath,' + os.path.dirname(lib)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    vals = dict(line.split(' ', 1) for line in out)
    from libcint_gb300 import molecules as M
    assert float(vals['norm']) == pytest.approx(M.gto_norm(2, 0.8), rel=1e-15)
    assert vals['sph'] == '1 10 cart 12 tot 11'       # d shell with two columns: 2 x 5 / 2 x 6
    assert int(vals['cache2e']) > 0 and int(vals['cache2c']) > 0
    assert vals['opt'] == '1' and vals['deleted'] == '1'
    assert vals['rc'].startswith('-1 msg') and 'ws_kb' in vals['rc']
    # the same arrays through ctypes give the same cache-size answers
    import ctypes
    atm = np.array([1, 20, 0, 0, 0, 0], np.int32)
    bas = np.array([0, 0, 2, 1, 0, 23, 25, 0, 0, 2, 1, 2, 0, 27, 28, 0], np.int32)
    env = np.zeros(40)
    env[23:25] = 1.3, 0.4
    env[25:27] = M.gto_norm(0, 1.3), M.gto_norm(0, 0.4)
    env[27:30] = 0.8, M.gto_norm(2, 0.8), 0.5 * M.gto_norm(2, 0.8)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    L = gpulib.lib()
    for name, shls, key in (('int2e_sph', [1, 0, 1, 1], 'cache2e'), ('int2c2e_sph', [1, 0], 'cache2c')):
        s = np.array(shls, np.int32)
        got = getattr(L, name)(None, None, P(s), P(atm), 1, P(bas), 2, P(env), None, None)
        assert got == int(vals[key]), (name, got, vals[key])


C_PLAN_SRC = r"""
#include <stddef.h>
#include <cuda_runtime.h>
#include "cintgpu.h"

/* the documented batched and J/K C usage, compiled and linked (not run: it needs a GPU) */
int run(const int *quartets, long n, const int *atm, int natm, const int *bas, int nbas,
        const double *env, double *out_dev, const double *dm_cart, double *xj, double *xk,
        size_t nao_cart, cudaStream_t stream)
{
    CINTGPUPlan *p;
    int rc = cintgpu_plan_create(&p, CINTGPU_INT2E_SPH, quartets, n, NULL, atm, natm, bas, nbas, env);
    if (rc) return rc;
    rc = cintgpu_plan_execute(p, out_dev, stream);
    cintgpu_plan_destroy(p);
    if (rc) return rc;
    rc = cintgpu_plan_create(&p, CINTGPU_JK_BUILD, quartets, n, NULL, atm, natm, bas, nbas, env);
    if (rc) return rc;
    cudaMemsetAsync(xj, 0, nao_cart * nao_cart * 8, stream);
    cudaMemsetAsync(xk, 0, nao_cart * nao_cart * 8, stream);
    rc = cintgpu_plan_execute_jk(p, dm_cart, xj, xk, stream);
    cintgpu_plan_destroy(p);
    return rc;
}

int main(void) { return 0; }
"""


def test_documented_plan_usage_compiles(gpulib, tmp_path):
    import shutil
    cc = shutil.which('gcc') or shutil.which('cc')
    cuda_inc = '/usr/local/cuda/include'
    if cc is None or not os.path.exists(os.path.join(cuda_inc, 'cuda_runtime.h')):
        pytest.skip('no C compiler or CUDA headers')
    lib = gpulib.lib()._name
    src = tmp_path / 'plans.c'
    src.write_text(C_PLAN_SRC)
    subprocess.run([cc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'), '-I', cuda_inc,
                    str(src), lib, '-L/usr/local/cuda/lib64', '-lcudart', '-o', str(tmp_path / 'plans'),
                    '-Wl,-rpath,' + os.path.dirname(lib)], check=True)
