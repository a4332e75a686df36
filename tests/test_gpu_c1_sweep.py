"""Element-wise parity on a class-stratified sample of the benchmark list (the committed c1 list:
120 atoms, 3s3p2d1f, 1-8 primitives; 55 kernel-order (li, lj, lk, ll) classes), batched plans on
the GPU against the CPU restatement and against its long-double build (the precision referee).

  absolute   up to 120 quartets of every class (6509): |diff| <= 1e-12 on every element of the
             int2e_sph and int2e_cart blocks, against the restatement;
  relative   up to 30 quartets of every class (1649): |diff| <= 1e-10 |ref| against the referee
             (every value in long double: x86 64-bit significand, aarch64 binary128) where
             |ref| > 1e-10 and |ref| > c of the quartet's largest Cartesian element; c = 1e-3 for
             Cartesian blocks (what the kernels compute) and 1e-2 for spherical ones.  Below c an
             element is the result of cancellation in the horizontal transfer or the cart -> sph
             transform and carries the block's absolute rounding: the transform of f shells
             cancels up to ~2e3 x, and libcint's own per-primitive algorithm (run on the GPU for
             (ff|ff)) leaves ~3.5e-12 of the Cartesian scale on some (ff|ff) elements, so the
             spherical elements between 1e-3 and 1e-2 of that scale reach 1e-9 for libcint's
             order of operations as well.
The double restatement is not the relative referee: it is itself off by up to 2e-9 on
uncancelled (ff|fs) Cartesian elements (its roots carry ~5e-15 of F0)."""
import numpy as np
import pytest

from libcint_gb300 import molecules as M
from tests import c1_sample

pytestmark = pytest.mark.gpu

ABS_TOL = 1e-12
REL_TOL = 1e-10
CUTOFF = {'int2e_cart': 1e-3, 'int2e_sph': 1e-2}


def gpu_blocks(gpulib, name, mol, qs):
    import torch
    kind = {'int2e_sph': gpulib.INT2E_SPH, 'int2e_cart': gpulib.INT2E_CART,
            'int2e_ip1_sph': gpulib.INT2E_IP1_SPH, 'int2e_ip1_cart': gpulib.INT2E_IP1_CART,
            'int3c2e_sph': gpulib.INT3C2E_SPH, 'int3c2e_cart': gpulib.INT3C2E_CART,
            'int2e_ip2_sph': gpulib.INT2E_IP2_SPH, 'int2e_ip2_cart': gpulib.INT2E_IP2_CART,
            'int3c2e_ip1_sph': gpulib.INT3C2E_IP1_SPH, 'int3c2e_ip1_cart': gpulib.INT3C2E_IP1_CART,
            'int3c2e_ip2_sph': gpulib.INT3C2E_IP2_SPH, 'int3c2e_ip2_cart': gpulib.INT3C2E_IP2_CART,
            'int2e_ipip1_sph': gpulib.INT2E_IPIP1_SPH, 'int2e_ipip1_cart': gpulib.INT2E_IPIP1_CART}[name]
    plan = gpulib.Plan(kind, mol, qs)
    out = torch.zeros(plan.output_size * plan.ncomp, dtype=torch.float64, device='cuda')
    plan.execute(out)
    res = out.cpu().numpy()
    plan.close()
    return res


def class_errors(got, ref, offs, cscale, classes, cutoff=1e-3):
    """per class: (max abs diff, max relative diff on elements above cutoff x the Cartesian scale)"""
    per = {}
    for q in range(len(offs) - 1):
        a, b = got[offs[q]:offs[q + 1]], ref[offs[q]:offs[q + 1]]
        d = np.abs(a - b)
        big = (np.abs(b) > 1e-10) & (np.abs(b) > cutoff * cscale[q])
        r = (d[big] / np.abs(b[big])).max(initial=0)
        key = tuple(int(x) for x in classes[q])
        e = per.get(key, (0.0, 0.0))
        per[key] = (max(e[0], d.max(initial=0)), max(e[1], r))
    return per


def cart_scales(oracle, mol, qs, ncomp=1):
    cart, offs = oracle.blocks('int2e_cart', mol, qs)
    return np.array([np.abs(cart[offs[q]:offs[q + 1]]).max(initial=0) for q in range(len(qs))])


@pytest.fixture(scope='module')
def c1():
    mol = M.config1(seed=0)
    return mol, c1_sample.c1_quartets()


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart'])
def test_c1_classes_absolute(gpulib, oracle, c1, name):
    mol, allq = c1
    qs, cls = c1_sample.stratified(mol, allq, 120)
    assert len(qs) >= 5000 and len(np.unique(cls, axis=0)) == 55
    ref, offs = oracle.blocks(name, mol, qs)
    got = gpu_blocks(gpulib, name, mol, qs)
    assert got.size == ref.size
    d = np.abs(got - ref)
    assert d.max() <= ABS_TOL, d.max()


@pytest.mark.parametrize('name', ['int2e_sph', 'int2e_cart'])
def test_c1_classes_relative(gpulib, oracle, c1, name):
    mol, allq = c1
    qs, cls = c1_sample.stratified(mol, allq, 30)
    ref, offs = oracle.referee(name, mol, qs)
    got = gpu_blocks(gpulib, name, mol, qs)
    per = class_errors(got, ref, offs, cart_scales(oracle, mol, qs), cls, CUTOFF[name])
    worst = max(per.items(), key=lambda kv: kv[1][1])
    print('%s: worst relative %.3e in class %s' % (name, worst[1][1], worst[0]))
    bad = {k: v for k, v in per.items() if v[1] > REL_TOL or v[0] > ABS_TOL}
    assert not bad, {k: ('%.2e' % v[0], '%.2e' % v[1]) for k, v in sorted(bad.items())}
