"""Shared-memory layouts of every class in every kernel mode, CPU only: what the kernels place in
a warp's shared memory (term records, g arrays, lane scratch, adjoint blocks) fits the budget the
planner launches them with, and the strides keep their bank-spreading properties."""
import ctypes

import pytest

from tests import _oracle  # noqa: F401  (puts the repo root on sys.path)
import libcint_gb300 as cg

ERI, IP1, GRAD, GRADA, ERIP, ERIB = 0, 1, 2, 3, 4, 5
TERMW, TERMW_GRAD, GRAD_MAXPRIM, W_SMEM = 12, 20, 16, 256
WS_SMALL, WS_MAX = 24 * 1024 // 8, 48 * 1024 // 8


class Layout(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ('lic nroots nmax mmax dI dJ dK dL G ng nf ncomp scr T off_dij off_dkl off_aacc '
                 'off_w off_g off_scr gstride gax termw').split()]


def layout(l, mode, ws):
    L = Layout()
    cg.lib().cg_layout(*l, mode, ws, ctypes.byref(L))
    return L


def nc(l):
    return (l + 1) * (l + 2) // 2


def classes(lmax):
    return [(a, b, c, d) for a in range(lmax + 1) for b in range(a + 1)
            for c in range(lmax + 1) for d in range(c + 1)]


# every shared-memory size per warp the regular group can be launched with (CINTGPU_WS_KB and the
# autotuner's candidates, 8..48 KB)
WS_ALL = [kb * 1024 // 8 for kb in (8, 12, 16, 20, 24, 28, 32, 40, 48)]


def test_bra_term_layouts_fit():
    """Bra-per-term classes: term records, the per-axis g(i, j, f) arrays (dI dJ (lk+ll+1), which
    hold the VRR array in place) and one VRR column of lane scratch per active lane fit."""
    for l in classes(6):
        if l[1] == 0:
            continue
        for ws in WS_ALL:
            L = layout(l, ERIB, ws)
            if L.T < 1:
                continue
            assert L.G == (l[0] + 1) * (l[1] + 1) * (l[2] + l[3] + 1)
            assert L.G >= (L.nmax + 1) * (L.mmax + 1)      # the VRR array fits in place
            assert L.gax % 2 == 1 and L.gax >= L.G and L.gstride == 3 * L.gax
            assert L.termw % 2 == 1 and L.termw >= 10 + L.mmax + 1
            assert L.scr % 2 == 1 and L.scr >= L.nmax + 1
            items = min(32, 3 * L.T)
            assert L.off_g == L.T * L.termw and L.off_scr == L.off_g + L.T * L.gstride
            assert L.off_scr + items * L.scr <= ws


@pytest.mark.parametrize('mode', [ERI, ERIP, IP1])
def test_integral_layouts_fit(mode):
    for l in classes(6):
        for ws in WS_ALL:
            L = layout(l, mode, ws)
            if L.T < 1:
                continue          # the planner rejects such a class or moves it to another group
            assert L.gax % 2 == 1 and L.gstride == 3 * L.gax
            if mode == ERI:
                assert L.termw % 2 == 1 and L.termw >= 10 + L.mmax + 1
                assert L.off_g == L.T * L.termw
                assert L.off_g + L.T * L.gstride <= ws
            else:
                assert L.scr % 2 == 1
                items = min(32, 3 * L.T)
                assert L.off_g == L.T * TERMW
                assert L.off_g + L.T * L.gstride + items * L.scr <= ws
                assert L.gax >= L.ng * L.G


# the exponent adjoint raises l by 2 on all four centres: these g-g / f-g classes exceed 48 KB
# per warp and the planner rejects them (CINTGPU_ERR_UNSUPPORTED)
GRADA_TOO_LARGE = {(3, 3, 4, 4), (4, 3, 4, 3), (4, 3, 4, 4), (4, 4, 3, 3), (4, 4, 4, 3), (4, 4, 4, 4)}


@pytest.mark.parametrize('mode', [GRAD, GRADA])
def test_adjoint_layouts_fit(mode):
    for l in classes(4):
        L = layout(l, mode, WS_MAX)
        if mode == GRADA and l in GRADA_TOO_LARGE:
            assert L.T < 1
            continue
        assert L.T >= 1, l
        assert L.gax % 2 == 1 and L.gstride == 3 * L.gax and L.scr % 2 == 1
        items = min(32, 3 * L.T)
        assert L.off_scr + items * L.scr <= WS_MAX
        assert L.off_g >= L.off_w and L.off_scr == L.off_g + L.T * L.gstride
        assert L.off_dkl - L.off_dij >= nc(l[0]) * nc(l[1])
        if mode == GRADA:
            assert L.off_w - L.off_aacc >= 4 * GRAD_MAXPRIM
        if L.nf <= W_SMEM:
            assert L.off_g - L.off_w >= L.nf


GRADJ, GRADAJ = 7, 8


def _np2(L):
    return 0 if L < 0 else (L + 1) * (L + 2) // 2


def _ntet(L):
    return 0 if L < 0 else (L + 1) * (L + 2) * (L + 3) // 6


@pytest.mark.parametrize('mode', [GRADJ, GRADAJ])
def test_contraction_first_adjoint_layouts_fit(mode):
    """Every l <= 4 class of the contraction-first adjoint fits 48 KB per warp: per-task densities
    (bra: the density, its i-weighted and AB-derivative transfers, 7 tetrahedra; ket: 4), the lane-owned sums (3 + 2 tetrahedra of the raised ranges; with
    exponents the four exponent weights and 64 per-primitive sums), then per term the record, the
    VRR arrays of both raised ranges and the larger side's contraction buffers (+ 64 exponent
    partials); strides odd."""
    ex = mode == GRADAJ
    d = 2 if ex else 1
    for l in classes(4):
        if l[0] * 16 + l[1] < l[2] * 16 + l[3]:
            continue                       # kernel order: the larger pair first
        L = layout(l, mode, WS_MAX)
        assert L.T >= 1, l
        Le, Lf = l[0] + l[1], l[2] + l[3]
        assert (L.nmax, L.mmax) == (Le + d, Lf + d)
        assert L.nroots == (sum(l) + d) // 2 + 1
        na, nm = L.nmax + 1, L.mmax + 1
        assert L.gax % 2 == 1 and L.gax >= na * nm and L.gstride == 3 * L.gax
        assert L.termw % 2 == 1 and L.termw >= 13 + nm + (2 if ex else 0)
        bufb = _np2(Lf) * na + (Lf + 1) * _np2(L.nmax)
        bufk = _np2(Le) * nm + (Le + 1) * _np2(L.mmax)
        assert L.scr >= max(bufb, bufk) + (64 if ex else 0) and L.scr % 2 == 1
        fixed = 7 * _ntet(Le) + 4 * _ntet(Lf) + 3 * _ntet(L.nmax) + 2 * _ntet(L.mmax)
        if ex:
            fixed += 2 * _ntet(L.nmax) + 2 * _ntet(L.mmax) + 4 * GRAD_MAXPRIM
        assert L.off_w == fixed and L.off_g == fixed + L.T * L.termw
        assert L.off_scr == L.off_g + L.T * L.gstride
        assert L.off_scr + L.T * L.scr <= WS_MAX
