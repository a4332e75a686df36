"""Coulomb-like contraction L = 1/2 sum D_ij (ij|kl) D_kl, its J matrix, the exchange matrix K,
and the hand-written adjoint exposed through torch.autograd.Function.

Forward: the CUDA kernels evaluate each unique shell quartet (i>=j, k>=l, ij>=kl) and contract it
with the density on the fly (J_BUILD, K_BUILD and JK_BUILD plans, the J/K build of a direct-SCF
driver); no (ij|kl) is stored.  Backward: the adjoint kernel
(J_GRAD / J_GRAD_EXP plans) recomputes Rys roots and g arrays with raised angular momenta and
returns dL/dR for every atom and, on request, dL/d(alpha) for every primitive exponent, at fixed
env coefficients.  dL/dD is J itself.  Comparator: `grad_via_ip1` forms int2e_ip1 blocks on the
same GPU (batched plans, written to HBM) and contracts them, the route libcint offers
(src/autocode/grad2.c:69-88).

Densities are spherical (libcint's int2e_sph AO order, contraction columns contiguous per shell).
"""
import ctypes

import numpy as np

from . import INT2E_IP1_SPH, _check, _ptr, lib
from .molecules import ANG_OF, ATOM_OF, NCTR_OF, NPRIM_OF, PTR_COORD, PTR_EXP, unique_quartets

J_BUILD, J_GRAD, J_GRAD_EXP, K_BUILD, JK_BUILD = 7, 8, 9, 10, 11


def cart2sph_matrix(mol):
    """Block-diagonal (nao_sph, nao_cart) matrix C with sph = C cart for every shell column."""
    L = lib()
    nsph = sum(mol.nsph(i) for i in range(mol.nbas))
    ncart = sum(mol.ncart(i) for i in range(mol.nbas))
    C = np.zeros((nsph, ncart))
    r = c = 0
    for i in range(mol.nbas):
        l = int(mol.bas[i, ANG_OF])
        nc = (l + 1) * (l + 2) // 2
        ns = 2 * l + 1 if l > 1 else nc
        blk = np.zeros(ns * nc)
        L.cintgpu_cart2sph(l, blk.ctypes.data_as(ctypes.c_void_p))
        blk = blk.reshape(ns, nc)
        for _ in range(int(mol.bas[i, NCTR_OF])):
            C[r:r + ns, c:c + nc] = blk
            r += ns
            c += nc
    return C


def _shell_diag_mask(mol, cart=True):
    loc = mol.ao_loc(cart=cart)
    n = loc[-1]
    m = np.zeros((n, n), dtype=bool)
    for i in range(mol.nbas):
        m[loc[i]:loc[i + 1], loc[i]:loc[i + 1]] = True
    return m


def exponents_of(mol):
    """All primitive exponents in shell order (the order of dL/d(alpha))."""
    return np.concatenate([mol.env[mol.bas[i, PTR_EXP]:mol.bas[i, PTR_EXP] + mol.bas[i, NPRIM_OF]]
                           for i in range(mol.nbas)])


def with_geometry(mol, coords=None, exps=None):
    """Copy of mol with atom coordinates (natm x 3, Bohr) and/or primitive exponents replaced."""
    m = mol.copy()
    if coords is not None:
        coords = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
        for a in range(m.natm):
            p = m.atm[a, PTR_COORD]
            m.env[p:p + 3] = coords[a]
    if exps is not None:
        exps = np.asarray(exps, dtype=np.float64).ravel()
        k = 0
        for i in range(m.nbas):
            p, n = m.bas[i, PTR_EXP], m.bas[i, NPRIM_OF]
            m.env[p:p + n] = exps[k:k + n]
            k += n
    return m


def atom_coords(mol):
    return np.array([mol.env[mol.atm[a, PTR_COORD]:mol.atm[a, PTR_COORD] + 3] for a in range(mol.natm)])


class _KindPlan:
    def __init__(self, kind, mol, quartets):
        L = lib()
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        h = ctypes.c_void_p()
        rc = L.cintgpu_plan_create(ctypes.byref(h), kind, _ptr(q), q.shape[0], None, _ptr(mol.atm),
                                   mol.natm, _ptr(mol.bas), mol.nbas, _ptr(mol.env))
        _check(rc, 'cintgpu_plan_create')
        self._h = h
        self.nao_cart = L.cintgpu_plan_nao_cart(h)
        self.flops = L.cintgpu_plan_flops(h)
        self.launches = L.cintgpu_plan_launches(h)

    def close(self):
        if getattr(self, '_h', None):
            lib().cintgpu_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream_ptr(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, 'cuda_stream') else int(stream))


class CoulombPlans:
    """Plans for one geometry: J and K contractions and (optionally) the adjoint."""

    def __init__(self, mol, quartets=None, with_exponents=False):
        import torch
        self.mol = mol
        self.quartets = unique_quartets(mol.nbas) if quartets is None else np.asarray(quartets)
        self.C = torch.as_tensor(cart2sph_matrix(mol), device='cuda')
        self.diag = torch.as_tensor(_shell_diag_mask(mol, cart=True), device='cuda')
        self.with_exponents = with_exponents
        self.jplan = _KindPlan(J_BUILD, mol, self.quartets)
        self.kplans = {}
        self.gplan = None

    def dm_cart(self, dm):
        return (self.C.T @ dm @ self.C).contiguous()

    def vj(self, dm, stream=None):
        """J (spherical) for the density dm (torch, cuda, float64, symmetric)."""
        return self.get_jk(dm, True, False, stream)[0]

    def vk(self, dm, stream=None):
        """K[i,k] = sum_jl (ij|kl) D[j,l] (spherical) for the symmetric density dm."""
        return self.get_jk(dm, False, True, stream)[1]

    def get_jk(self, dm, with_j=True, with_k=True, stream=None):
        """(J, K) for the symmetric density dm (None for the one not asked); with both, each
        quartet is evaluated once and contracted into both."""
        import torch
        if not (with_j or with_k):
            return None, None
        kind = JK_BUILD if (with_j and with_k) else (J_BUILD if with_j else K_BUILD)
        if kind == J_BUILD:
            plan = self.jplan
        else:
            if kind not in self.kplans:
                self.kplans[kind] = _KindPlan(kind, self.mol, self.quartets)
            plan = self.kplans[kind]
        dmc = self.dm_cart(dm)
        XJ = torch.zeros_like(dmc) if with_j else None
        XK = torch.zeros_like(dmc) if with_k else None
        ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        _check(lib().cintgpu_plan_execute_jk(plan._h, ptr(dmc), ptr(XJ), ptr(XK), _stream_ptr(stream)),
               'cintgpu_plan_execute_jk')
        J = K = None
        if with_j:
            J = self.C @ (XJ + XJ.T - torch.where(self.diag, XJ, torch.zeros_like(XJ))) @ self.C.T
        if with_k:
            K = self.C @ (XK + XK.T) @ self.C.T
        return J, K

    def energy(self, dm, stream=None):
        J = self.vj(dm, stream)
        return 0.5 * (dm * J).sum(), J

    def grad(self, dm, stream=None):
        """(dL/dR (natm, 3), dL/dalpha or None) for L = 1/2 D (ij|kl) D."""
        import torch
        if self.gplan is None:
            self.gplan = _KindPlan(J_GRAD_EXP if self.with_exponents else J_GRAD, self.mol,
                                   self.quartets)
        dmc = self.dm_cart(dm)
        g = torch.zeros((self.mol.natm, 3), dtype=torch.float64, device='cuda')
        ga = None
        if self.with_exponents:
            ga = torch.zeros(int(self.mol.bas[:, NPRIM_OF].sum()), dtype=torch.float64, device='cuda')
        _check(lib().cintgpu_plan_execute_grad(self.gplan._h, ctypes.c_void_p(dmc.data_ptr()),
                                               ctypes.c_void_p(g.data_ptr()),
                                               None if ga is None else ctypes.c_void_p(ga.data_ptr()),
                                               _stream_ptr(stream)), 'cintgpu_plan_execute_grad')
        return g, ga


def _autograd_function():
    import torch

    class CoulombEnergy(torch.autograd.Function):
        """L = 1/2 sum D_ij (ij|kl) D_kl as a differentiable function of atom coordinates
        (natm x 3, Bohr), primitive exponents (shell order) and the spherical density."""

        @staticmethod
        def forward(ctx, coords, exps, dm, mol, quartets):
            m = with_geometry(mol, coords.detach().cpu().numpy(), exps.detach().cpu().numpy())
            plans = CoulombPlans(m, quartets, with_exponents=exps.requires_grad)
            dmd = dm.detach()
            E, J = plans.energy(dmd)
            ctx.plans = plans
            ctx.devs = (coords.device, exps.device)
            ctx.save_for_backward(dmd, J)
            return E

        @staticmethod
        def backward(ctx, gE):
            dm, J = ctx.saved_tensors
            plans = ctx.plans
            g, ga = plans.grad(dm)
            gc = (gE * g).to(ctx.devs[0]) if ctx.needs_input_grad[0] else None
            gx = (gE * ga).to(ctx.devs[1]) if (ga is not None and ctx.needs_input_grad[1]) else None
            gd = (gE * J) if ctx.needs_input_grad[2] else None
            return gc, gx, gd, None, None

    return CoulombEnergy


_CE = None


def coulomb_energy(coords, exps, dm, mol, quartets=None):
    """Differentiable L(coords, exps, dm) = 1/2 sum D (ij|kl) D (torch tensors on cuda)."""
    global _CE
    if _CE is None:
        _CE = _autograd_function()
    return _CE.apply(coords, exps, dm, mol, quartets)


class _IP1Pass:
    """One pass of the comparator: int2e_ip1_sph blocks of the quartets in shell order perm (the
    derivative on the first shell), formed by one batched GPU plan (class-contiguous offsets) and
    contracted with -1/2 w D_ij D_kl per quartet.  The plan and the index tensors are built at
    construction; run() only executes and contracts."""

    def __init__(self, mol, q, w, perm):
        import torch
        from . import Plan
        loc = mol.ao_loc()
        ls = mol.bas[:, ANG_OF]
        qq = np.ascontiguousarray(q[:, perm])
        key = ls[qq[:, 0]] * 1000 + ls[qq[:, 1]] * 100 + ls[qq[:, 2]] * 10 + ls[qq[:, 3]]
        order = np.argsort(key, kind='stable')
        qs, ws = qq[order], w[order]
        d = np.array([mol.nsph(s) for s in range(mol.nbas)])
        sizes = d[qs[:, 0]] * d[qs[:, 1]] * d[qs[:, 2]] * d[qs[:, 3]]
        offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        self.plan = Plan(INT2E_IP1_SPH, mol, qs, offs)
        self.out = torch.empty(3 * self.plan.output_size, dtype=torch.float64, device='cuda')
        self.n = len(qs)
        ks = key[order]
        bounds = np.flatnonzero(np.diff(ks)) + 1
        self.segs = []
        for seg in np.split(np.arange(len(qs)), bounds):
            if len(seg) == 0:
                continue
            a, b, c, e = (int(d[qs[seg[0], x]]) for x in range(4))
            t = lambda v: torch.as_tensor(v, device='cuda')
            self.segs.append((int(offs[seg[0]]), len(seg), (a, b, c, e),
                              t(loc[qs[seg, 0]][:, None] + np.arange(a)[None]),
                              t(loc[qs[seg, 1]][:, None] + np.arange(b)[None]),
                              t(loc[qs[seg, 2]][:, None] + np.arange(c)[None]),
                              t(loc[qs[seg, 3]][:, None] + np.arange(e)[None]),
                              t(ws[seg]), t(seg)))
        self.order = torch.as_tensor(order, device='cuda')

    def run(self, dmd):
        import torch
        self.plan.execute(self.out)
        out = self.out.view(3, self.plan.output_size)
        res = torch.empty((self.n, 3), dtype=torch.float64, device='cuda')
        for off, n, (a, b, c, e), ii, jj, kk, ll, wt, seg in self.segs:
            blk = out[:, off:off + n * a * b * c * e].reshape(3, n, e, c, b, a)  # i fastest
            Dij = dmd[ii[:, :, None], jj[:, None, :]]
            Dkl = dmd[kk[:, :, None], ll[:, None, :]]
            res[seg] = torch.einsum('xnlkji,nij,nkl,n->nx', blk, Dij, Dkl, wt) * -0.5
        back = torch.empty_like(res)
        back[self.order] = res
        return back

    def close(self):
        self.plan.close()


class IP1Gradient:
    """dL/dR from int2e_ip1 integrals formed on the GPU (written to HBM, batched plans) and
    contracted with the density: the comparator route, libcint's (src/autocode/grad2.c:69-88).
    Three passes over the unique quartet list put the derivative on i, j and k ((ij|kl), (ji|kl),
    (kl|ij)); the fourth centre follows from translational invariance, per quartet.  The plans
    are built once at construction, like the adjoint's."""

    def __init__(self, mol, quartets=None):
        import torch
        q = unique_quartets(mol.nbas) if quartets is None else np.asarray(quartets, dtype=np.int32)
        self.mol = mol
        w = (np.where(q[:, 0] != q[:, 1], 2.0, 1.0) * np.where(q[:, 2] != q[:, 3], 2.0, 1.0)
             * np.where((q[:, 0] != q[:, 2]) | (q[:, 1] != q[:, 3]), 2.0, 1.0))
        self.passes = [_IP1Pass(mol, q, w, perm) for perm in ((0, 1, 2, 3), (1, 0, 2, 3), (2, 3, 0, 1))]
        atom = mol.bas[:, ATOM_OF]
        self.atoms = [torch.as_tensor(atom[q[:, col]], device='cuda') for col in range(4)]

    def grad(self, dm):
        import torch
        dmd = dm.detach()
        vi, vj, vk = (p.run(dmd) for p in self.passes)
        vl = -(vi + vj + vk)
        grad = torch.zeros((self.mol.natm, 3), dtype=torch.float64, device='cuda')
        for col, v in enumerate((vi, vj, vk, vl)):
            grad.index_add_(0, self.atoms[col], v)
        return grad

    def close(self):
        for p in self.passes:
            p.close()


def grad_via_ip1(mol, dm, quartets=None):
    """dL/dR through the int2e_ip1 route (IP1Gradient), plans built and released in the call."""
    r = IP1Gradient(mol, quartets)
    try:
        return r.grad(dm)
    finally:
        r.close()
