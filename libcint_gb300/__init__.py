"""libcint_gb300 -- GB300-native Rys-quadrature two-electron integrals behind libcint's C API.

The product is the C-ABI library libcintgpu.so (include/cintgpu.h).  This package builds it,
loads it with ctypes, and adds the thin Python layer the autograd wrapper needs.  There is no
CPU fallback: every call goes through the CUDA kernels, and a missing library is an error.
"""
import ctypes
import os

import numpy as np

from .build import LIB as _LIB_PATH, build, build_library  # noqa: F401
from . import molecules  # noqa: F401

INT2E_SPH, INT2E_CART, INT2E_IP1_SPH, INT2E_IP1_CART, INT3C2E_SPH, INT3C2E_CART = 1, 2, 3, 4, 5, 6
INT2C2E_SPH, INT2C2E_CART = 12, 13
INT2E_IP2_SPH, INT2E_IP2_CART = 14, 15
INT3C2E_IP1_SPH, INT3C2E_IP1_CART, INT3C2E_IP2_SPH, INT3C2E_IP2_CART = 16, 17, 18, 19
INT2E_IPIP1_SPH, INT2E_IPIP1_CART = 20, 21
_KIND_NSH = {1: 4, 2: 4, 3: 4, 4: 4, 5: 3, 6: 3, 12: 2, 13: 2, 14: 4, 15: 4, 16: 3, 17: 3, 18: 3, 19: 3,
             20: 4, 21: 4}

_lib = None


class CintGpuError(RuntimeError):
    pass


def lib():
    """The loaded libcintgpu.so (built on first use if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build_library()
    if not os.path.exists(_LIB_PATH):
        raise CintGpuError('libcintgpu.so is missing and could not be built: ' + _LIB_PATH)
    L = ctypes.CDLL(_LIB_PATH)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    for name in ('int2e_sph', 'int2e_cart', 'int2e_ip1_sph', 'int2e_ip1_cart', 'int3c2e_sph',
                 'int3c2e_cart', 'int2c2e_sph', 'int2c2e_cart', 'int2e_ip2_sph', 'int2e_ip2_cart',
                 'int3c2e_ip1_sph', 'int3c2e_ip1_cart', 'int3c2e_ip2_sph', 'int3c2e_ip2_cart',
                 'int2e_ipip1_sph', 'int2e_ipip1_cart'):
        f = getattr(L, name)
        f.restype = i32
        f.argtypes = [vp, vp, vp, vp, i32, vp, i32, vp, vp, vp]
    for name in ('cint2e_sph', 'cint2e_cart', 'cint2e_ip1_sph', 'cint2e_ip1_cart', 'cint3c2e_sph',
                 'cint3c2e_cart', 'cint2c2e_sph', 'cint2c2e_cart', 'cint2e_ip2_sph',
                 'cint2e_ip2_cart', 'cint3c2e_ip1_sph', 'cint3c2e_ip1_cart', 'cint3c2e_ip2_sph',
                 'cint3c2e_ip2_cart', 'cint2e_ipip1_sph', 'cint2e_ipip1_cart'):
        f = getattr(L, name)
        f.restype = i32
        f.argtypes = [vp, vp, vp, i32, vp, i32, vp, vp]
    for name in ('int2e_optimizer', 'int2e_ip1_optimizer', 'int3c2e_optimizer', 'int2c2e_optimizer',
                 'int2e_ip2_optimizer', 'int3c2e_ip1_optimizer', 'int3c2e_ip2_optimizer',
                 'int2e_ipip1_optimizer'):
        f = getattr(L, name)
        f.restype = None
        f.argtypes = [vp, vp, i32, vp, i32, vp]
    L.CINTdel_optimizer.argtypes = [vp]
    L.CINTdel_optimizer.restype = None
    L.CINTgto_norm.argtypes = [i32, dbl]
    L.CINTgto_norm.restype = dbl
    L.cintgpu_plan_create.argtypes = [vp, i32, vp, i64, vp, vp, i32, vp, i32, vp]
    L.cintgpu_plan_create.restype = i32
    L.cintgpu_plan_create_tuned.argtypes = [vp, i32, vp, i64, vp, vp, i32, vp, i32, vp, i32, i32]
    L.cintgpu_plan_create_tuned.restype = i32
    L.cintgpu_plan_create_classes.argtypes = [vp, i32, vp, i64, vp, vp, i32, vp, i32, vp, i32, i32, vp, i32]
    L.cintgpu_plan_create_classes.restype = i32
    L.cintgpu_plan_output_size.argtypes = [vp]
    L.cintgpu_plan_output_size.restype = i64
    L.cintgpu_plan_ncomp.argtypes = [vp]
    L.cintgpu_plan_ncomp.restype = i32
    L.cintgpu_plan_flops.argtypes = [vp]
    L.cintgpu_plan_flops.restype = dbl
    L.cintgpu_plan_prim_quartets.argtypes = [vp]
    L.cintgpu_plan_prim_quartets.restype = i64
    L.cintgpu_plan_upload_bytes.argtypes = [vp]
    L.cintgpu_plan_upload_bytes.restype = i64
    L.cintgpu_plan_launches.argtypes = [vp]
    L.cintgpu_plan_launches.restype = i32
    L.cintgpu_plan_flops_libcint.argtypes = [vp]
    L.cintgpu_plan_flops_libcint.restype = ctypes.c_double
    L.cintgpu_plan_compute_ms.argtypes = [vp]
    L.cintgpu_plan_compute_ms.restype = ctypes.c_float
    L.cintgpu_plan_execute.argtypes = [vp, vp, vp]
    L.cintgpu_plan_execute.restype = i32
    L.cintgpu_plan_nonempty.argtypes = [vp, vp]
    L.cintgpu_plan_nonempty.restype = i32
    L.cintgpu_plan_destroy.argtypes = [vp]
    L.cintgpu_plan_destroy.restype = None
    L.cintgpu_batch_host.argtypes = [i32, vp, vp, i64, vp, vp, i32, vp, i32, vp]
    L.cintgpu_batch_host.restype = i32
    L.cintgpu_batch_device.argtypes = [i32, vp, vp, i64, vp, i32, vp, i32, vp]
    L.cintgpu_batch_device.restype = i32
    L.cintgpu_rys_roots_dev.argtypes = [i32, vp, i32, vp, vp, vp]
    L.cintgpu_rys_roots_dev.restype = i32
    L.cintgpu_rys_nmax.restype = i32
    L.cintgpu_plan_status.argtypes = [vp]
    L.cintgpu_plan_status.restype = i32
    L.cintgpu_plan_nao_cart.argtypes = [vp]
    L.cintgpu_plan_nao_cart.restype = i32
    L.cintgpu_plan_execute_j.argtypes = [vp, vp, vp, vp]
    L.cintgpu_plan_execute_j.restype = i32
    L.cintgpu_plan_execute_jk.argtypes = [vp, vp, vp, vp, vp]
    L.cintgpu_plan_execute_jk.restype = i32
    L.cintgpu_plan_execute_grad.argtypes = [vp, vp, vp, vp, vp]
    L.cintgpu_plan_execute_grad.restype = i32
    L.cintgpu_cart2sph.argtypes = [i32, vp]
    L.cintgpu_cart2sph.restype = i32
    L.cintgpu_last_error.restype = ctypes.c_char_p
    L.cintgpu_screened_run.restype = i32
    L.cintgpu_screened_run.argtypes = [i32, vp, vp, i64, dbl, i64, i64, vp, i32, vp, i32, vp, vp, vp,
                                       vp, vp, vp, vp]
    L.cintgpu_dropin_failures.restype = i64
    L.cintgpu_dropin_failures.argtypes = []
    L.cintgpu_device_sm_count.restype = i32
    L.cintgpu_df_create.argtypes = [vp, vp, i64, i32, i32]
    L.cintgpu_df_create.restype = i32
    L.cintgpu_df_size.argtypes = [vp]
    L.cintgpu_df_size.restype = i64
    L.cintgpu_df_rho.argtypes = [vp, vp, vp, vp, vp]
    L.cintgpu_df_rho.restype = i32
    L.cintgpu_df_j.argtypes = [vp, vp, vp, vp, vp]
    L.cintgpu_df_j.restype = i32
    L.cintgpu_df_destroy.argtypes = [vp]
    L.cintgpu_df_destroy.restype = None
    _lib = L
    return L


def last_error():
    return lib().cintgpu_last_error().decode()


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise CintGpuError('%s failed (%d): %s' % (what, rc, last_error()))


class Plan:
    """A batched evaluation plan: n items (shell quartets; triples for int3c2e, pairs for int2c2e)
    of one kind.

    execute(out) enqueues the kernels writing into a CUDA float64 buffer (a torch tensor or a raw
    device pointer) of ncomp * output_size elements; block q of component c starts at
    c * output_size + offsets[q] and is laid out like libcint's dense output (i fastest).
    ws_kb / separate_output: the launch parameters of cintgpu_plan_create_tuned (0 = defaults);
    wide_classes: class keys ((li*8 + lj)*8 + lk)*8 + ll, kernel order) run with 48 KB of shared
    memory per warp (cintgpu_plan_create_classes); autotune.tuned_plan picks all three."""

    def __init__(self, kind, mol, shls, offsets=None, ws_kb=0, separate_output=0, wide_classes=()):
        L = lib()
        self.kind = kind
        self.mol = mol
        shls = np.ascontiguousarray(shls, dtype=np.int32).reshape(-1, _KIND_NSH[kind])
        self.n = shls.shape[0]
        off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.int64)
        h = ctypes.c_void_p()
        args = (ctypes.byref(h), kind, _ptr(shls), self.n, _ptr(off), _ptr(mol.atm), mol.natm,
                _ptr(mol.bas), mol.nbas, _ptr(mol.env))
        wide = np.ascontiguousarray(sorted(set(int(k) for k in wide_classes)), dtype=np.int32)
        if len(wide):
            rc = L.cintgpu_plan_create_classes(*args, int(ws_kb), int(separate_output), _ptr(wide),
                                               len(wide))
        elif ws_kb or separate_output:
            rc = L.cintgpu_plan_create_tuned(*args, int(ws_kb), int(separate_output))
        else:
            rc = L.cintgpu_plan_create(*args)
        _check(rc, 'cintgpu_plan_create')
        self.ws_kb, self.separate_output = int(ws_kb), int(separate_output)
        self.wide_classes = tuple(int(k) for k in wide)
        self._h = h
        self.output_size = L.cintgpu_plan_output_size(h)
        self.ncomp = L.cintgpu_plan_ncomp(h)
        self.flops = L.cintgpu_plan_flops(h)
        self.flops_libcint = L.cintgpu_plan_flops_libcint(h)
        self.prim_quartets = L.cintgpu_plan_prim_quartets(h)
        self.launches = L.cintgpu_plan_launches(h)

    def execute(self, out, stream=None):
        ptr = out.data_ptr() if hasattr(out, 'data_ptr') else int(out)
        if hasattr(out, 'numel'):
            if out.numel() < self.ncomp * self.output_size or str(out.dtype) != 'torch.float64' \
                    or not out.is_cuda:
                raise CintGpuError('output must be a CUDA float64 tensor of >= %d elements'
                                   % (self.ncomp * self.output_size))
        st = None
        if stream is not None:
            st = ctypes.c_void_p(stream.cuda_stream if hasattr(stream, 'cuda_stream') else int(stream))
        _check(lib().cintgpu_plan_execute(self._h, ctypes.c_void_p(ptr), st), 'cintgpu_plan_execute')

    def nonempty(self):
        flags = np.zeros(self.n, dtype=np.int32)
        _check(lib().cintgpu_plan_nonempty(self._h, _ptr(flags)), 'cintgpu_plan_nonempty')
        return flags

    def compute_ms(self):
        """Device time of the last execution's integral kernels (output transform excluded),
        from CUDA events on its stream; synchronises."""
        return float(lib().cintgpu_plan_compute_ms(self._h))

    def close(self):
        if getattr(self, '_h', None):
            lib().cintgpu_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_host(kind, mol, shls, offsets=None):
    """One-shot host-buffer evaluation: returns (ncomp, output_size) float64 numpy array."""
    shls = np.ascontiguousarray(shls, dtype=np.int32).reshape(-1, _KIND_NSH.get(kind, 4))
    sph = kind in (INT2E_SPH, INT2E_IP1_SPH, INT3C2E_SPH, INT2C2E_SPH)
    ncomp = 3 if kind in (INT2E_IP1_SPH, INT2E_IP1_CART) else 1
    per = np.array([mol.nsph(s) if sph else mol.ncart(s) for s in range(mol.nbas)], dtype=np.int64)
    blocks = np.prod(per[shls], axis=1) if len(shls) else np.zeros(0, np.int64)
    if offsets is None:
        size = int(blocks.sum())
    else:
        size = int((np.asarray(offsets, dtype=np.int64) + blocks).max(initial=0))
    out = np.zeros(ncomp * size)
    off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.int64)
    rc = lib().cintgpu_batch_host(kind, _ptr(out), _ptr(shls), shls.shape[0], _ptr(off),
                                  _ptr(mol.atm), mol.natm, _ptr(mol.bas), mol.nbas, _ptr(mol.env))
    _check(rc, 'cintgpu_batch_host')
    return out.reshape(ncomp, size)


def batch_device(kind, mol, shls, out):
    """cintgpu_batch_device: the blocks of one-component kinds straight into the CUDA float64
    tensor out (back to back, libcint's layout per block), chunks planned on host threads while
    the GPU runs earlier ones; returns when done."""
    shls = np.ascontiguousarray(shls, dtype=np.int32).reshape(-1, _KIND_NSH[kind])
    _check(lib().cintgpu_batch_device(kind, ctypes.c_void_p(out.data_ptr()), _ptr(shls), shls.shape[0],
                                      _ptr(mol.atm), mol.natm, _ptr(mol.bas), mol.nbas, _ptr(mol.env)),
           'cintgpu_batch_device')


def dropin(name, mol, shls, dims=None, nbas=None):
    """Call one libcint-signature entry point of libcintgpu (e.g. 'int2e_sph') for one shell
    block; returns (flag, out) with out the dense block (Fortran order, components last)."""
    L = lib()
    f = getattr(L, name)
    nsh = 3 if 'int3c2e' in name else (2 if 'int2c2e' in name else 4)
    shls = np.ascontiguousarray(shls, dtype=np.int32)
    sph = name.endswith('_sph')
    ncomp = 9 if '_ipip1' in name else (3 if ('_ip1' in name or '_ip2' in name) else 1)
    cnt = [(mol.nsph(s) if sph else mol.ncart(s)) for s in shls[:nsh]]
    n = int(np.prod(cnt)) * ncomp
    out = np.zeros(n if dims is None else int(np.prod(dims)) * ncomp)
    d = None if dims is None else np.ascontiguousarray(dims, dtype=np.int32)
    flag = f(_ptr(out), _ptr(d), _ptr(shls), _ptr(mol.atm), mol.natm, _ptr(mol.bas),
             mol.nbas if nbas is None else nbas, _ptr(mol.env), None, None)
    if dims is None:
        return flag, out.reshape(cnt + ([ncomp] if ncomp > 1 else []), order='F')
    return flag, out


def rys_roots(nroots, xs):
    """Rys nodes s = t^2 and weights from the device tables (testing aid); needs torch + CUDA."""
    import torch
    x = torch.as_tensor(np.ascontiguousarray(xs, dtype=np.float64), device='cuda')
    s = torch.empty((x.numel(), nroots), dtype=torch.float64, device='cuda')
    w = torch.empty_like(s)
    _check(lib().cintgpu_rys_roots_dev(nroots, ctypes.c_void_p(x.data_ptr()), x.numel(),
                                       ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                       None), 'cintgpu_rys_roots_dev')
    torch.cuda.synchronize()
    return s.cpu().numpy(), w.cpu().numpy()
