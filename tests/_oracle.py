"""Loader for the CPU oracle libraries (tests only).

liboracle.so is the C restatement in oracle/ (always built); libcint.so is the reference itself,
compiled from its sources into oracle/_ref/ where those sources exist (not on every machine).
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ODIR = os.path.join(ROOT, 'oracle')
ORACLE_SO = os.path.join(ODIR, '_build', 'liboracle.so')
ORACLE_LD_SO = os.path.join(ODIR, '_build', 'liboracle_ld.so')
REF_SO = os.path.join(ODIR, '_ref', 'libcint.so')

_SIG = ('int2e_sph', 'int2e_cart', 'int2e_ip1_sph', 'int2e_ip1_cart', 'int3c2e_sph', 'int3c2e_cart',
        'int2c2e_sph', 'int2c2e_cart', 'int2e_ip2_sph', 'int2e_ip2_cart', 'int3c2e_ip1_sph',
        'int3c2e_ip1_cart', 'int3c2e_ip2_sph', 'int3c2e_ip2_cart', 'int2e_ipip1_sph',
        'int2e_ipip1_cart')


class _Lib:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        for name in _SIG:
            f = getattr(self.lib, prefix + name)
            f.restype = i32
            f.argtypes = [vp, vp, vp, vp, i32, vp, i32, vp, vp, vp]

    def call(self, name, mol, shls, dims=None, nbas=None):
        f = getattr(self.lib, self.prefix + name)
        nsh = 3 if 'int3c2e' in name else (2 if 'int2c2e' in name else 4)
        shls = np.ascontiguousarray(shls, dtype=np.int32)
        sph = name.endswith('_sph')
        ncomp = 9 if '_ipip1' in name else (3 if ('_ip1' in name or '_ip2' in name) else 1)
        cnt = [(mol.nsph(s) if sph else mol.ncart(s)) for s in shls[:nsh]]
        n = int(np.prod(cnt)) * ncomp
        out = np.zeros(n if dims is None else int(np.prod(dims)) * ncomp)
        P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
        d = None if dims is None else np.ascontiguousarray(dims, dtype=np.int32)
        flag = f(P(out), P(d), P(shls), P(mol.atm), mol.natm, P(mol.bas),
                 mol.nbas if nbas is None else nbas, P(mol.env), None, None)
        if dims is None:
            return flag, out.reshape(cnt + ([ncomp] if ncomp > 1 else []), order='F')
        return flag, out


class Oracles:
    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            subprocess.run(['make', '-s', '-C', ODIR, 'oracle'], check=True)
        self.port = _Lib(ORACLE_SO, 'oracle_')
        self.port.lib.oracle_rys_roots.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                                                   ctypes.c_void_p]
        self.port.lib.oracle_rys_roots.restype = ctypes.c_int
        self.ld = None
        self.ref = _Lib(REF_SO, '') if os.path.exists(REF_SO) else None
        if self.ref is not None:
            L = self.ref.lib
            L.CINTrys_roots.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
            L.CINTrys_roots.restype = None

    KINDS = _SIG

    def blocks(self, name, mol, items, threads=0):
        """Dense blocks of many items through the restatement, OpenMP over items (oracle_list).
        Returns (flat, offsets): item q's block (all components, libcint layout) is
        flat[offsets[q]:offsets[q + 1]]."""
        which = self.KINDS.index(name)
        nsh = 3 if 'int3c2e' in name else (2 if 'int2c2e' in name else 4)
        items = np.ascontiguousarray(items, dtype=np.int32).reshape(-1, nsh)
        sph = name.endswith('_sph')
        ncomp = 9 if '_ipip1' in name else (3 if ('_ip1' in name or '_ip2' in name) else 1)
        l = mol.bas[:, 1].astype(np.int64)
        nctr = mol.bas[:, 3].astype(np.int64)
        per = ((2 * l + 1) if sph else (l + 1) * (l + 2) // 2) * nctr
        size = np.prod(per[items], axis=1) * ncomp
        offs = np.concatenate([[0], np.cumsum(size)]).astype(np.int64)
        out = np.zeros(int(offs[-1]))
        L = self.port.lib
        L.oracle_list.restype = ctypes.c_double
        vp = ctypes.c_void_p
        L.oracle_list.argtypes = [ctypes.c_int, vp, ctypes.c_long, vp, vp, vp, ctypes.c_int, vp,
                                  ctypes.c_int, vp, ctypes.c_int]
        P = lambda a: a.ctypes.data_as(vp)
        t = L.oracle_list(which, P(items), len(items), P(out), P(offs), P(mol.atm), mol.natm,
                          P(mol.bas), mol.nbas, P(mol.env), threads)
        assert t >= 0
        return out, offs

    def referee(self, name, mol, items, threads=0):
        """The same blocks as blocks(), computed by the long-double build of the restatement
        (liboracle_ld.so: every value, the inputs included, in long double); returned as
        float64 (flat, offsets).  The precision referee for relative-accuracy gates."""
        if self.ld is None:
            self.ld = ctypes.CDLL(ORACLE_LD_SO)
        which = self.KINDS.index(name)
        nsh = 3 if 'int3c2e' in name else (2 if 'int2c2e' in name else 4)
        items = np.ascontiguousarray(items, dtype=np.int32).reshape(-1, nsh)
        sph = name.endswith('_sph')
        ncomp = 9 if '_ipip1' in name else (3 if ('_ip1' in name or '_ip2' in name) else 1)
        l = mol.bas[:, 1].astype(np.int64)
        nctr = mol.bas[:, 3].astype(np.int64)
        per = ((2 * l + 1) if sph else (l + 1) * (l + 2) // 2) * nctr
        size = np.prod(per[items], axis=1) * ncomp
        offs = np.concatenate([[0], np.cumsum(size)]).astype(np.int64)
        out = np.zeros(int(offs[-1]), dtype=np.longdouble)
        env = np.ascontiguousarray(mol.env, dtype=np.longdouble)
        f = self.ld.oracle_ld_list
        f.restype = ctypes.c_longdouble
        vp = ctypes.c_void_p
        f.argtypes = [ctypes.c_int, vp, ctypes.c_long, vp, vp, vp, ctypes.c_int, vp, ctypes.c_int,
                      vp, ctypes.c_int]
        P = lambda a: a.ctypes.data_as(vp)
        t = f(which, P(items), len(items), P(out), P(offs), P(mol.atm), mol.natm, P(mol.bas),
              mol.nbas, P(env), threads)
        assert t >= 0
        return out.astype(np.float64), offs

    def roots(self, n, x):
        u = np.zeros(n)
        w = np.zeros(n)
        rc = self.port.lib.oracle_rys_roots(n, float(x), u.ctypes.data_as(ctypes.c_void_p),
                                            w.ctypes.data_as(ctypes.c_void_p))
        assert rc == 0
        return u / (1 + u), w


_cached = None


def load():
    global _cached
    if _cached is None:
        _cached = Oracles()
    return _cached
