"""Gradient harness: chains of coagulation + condensation steps on the GPU.

`SalsaChain` drives the chain entry points of the C-ABI (salsa_gb300_chain_*):
the forward chain with per-step checkpoints, its tangent-linear model, and the
hand-written adjoint.  `chain_apply` wraps them in a torch.autograd.Function, so
gradients of any function of the final bin state with respect to the initial bin
state, kappa and the imposed supersaturation come from the adjoint kernel.

State layout per cell (nstate = nliquid * (1 + nwet)): the numbers of the liquid
bins [#/kg] (aerosol, cloud, precipitation), then the masses m[s][b] [kg/kg],
species-major with the liquid bins fastest.  A step is the coagulation
(mo_salsa_dynamics.f90:92-202) followed by the water condensation
(mo_salsa_dynamics.f90:691-1125) of a warm cell with empty precipitation bins; the
vapour is reset to rs (1 + s) at the start of every step.
"""
import ctypes as C

import torch

from . import api
from .capi import SALSA_OK, ERROR_NAMES
from .config import workload_config

_PD = C.POINTER(C.c_double)


class ChainDesc(C.Structure):
    _fields_ = [("ncell", C.c_int), ("nsub", C.c_int), ("dt", C.c_double),
                ("temp", _PD), ("press", _PD), ("rs", _PD), ("dn", _PD), ("kappa", _PD), ("ssat", _PD)]


def _p(t):
    if t is None:
        return _PD()
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError("chain arrays must be contiguous float64 CUDA tensors")
    return C.cast(C.c_void_p(t.data_ptr()), _PD)


def chain_config():
    """Level-4 configuration of the chain: coagulation and condensation on, the
    processes the chain leaves out (autoconversion, activation, redistribution) off."""
    c = workload_config(level=4, precision=0, diagnostics=0)
    c.lsauto.sw = 0
    c.lsactiv.sw = 0
    c.lsdistupdate = 0
    return c


def _lib():
    L = api.library()
    if not hasattr(L, "_chain_ready"):
        L.salsa_gb300_chain_state_size.argtypes = [C.c_void_p]
        L.salsa_gb300_chain_state_size.restype = C.c_int
        L.salsa_gb300_chain_adjoint_bytes.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int]
        L.salsa_gb300_chain_adjoint_bytes.restype = C.c_longlong
        L.salsa_gb300_chain_forward.argtypes = [C.c_void_p, C.POINTER(ChainDesc), _PD, _PD, _PD, C.c_int, C.c_void_p]
        L.salsa_gb300_chain_tlm.argtypes = [C.c_void_p, C.POINTER(ChainDesc), _PD, _PD, _PD, _PD, _PD, _PD,
                                            C.c_void_p]
        L.salsa_gb300_chain_adjoint.argtypes = [C.c_void_p, C.POINTER(ChainDesc), _PD, C.c_int, _PD, _PD, _PD, _PD,
                                                C.c_void_p]
        for f in ("salsa_gb300_chain_forward", "salsa_gb300_chain_tlm", "salsa_gb300_chain_adjoint"):
            getattr(L, f).restype = C.c_int
        L._chain_ready = True
    return L


class SalsaChain:
    """Chains of nsub steps of length dt over independent cells (one level-4 handle)."""

    def __init__(self, cfg=None):
        self.step = api.SalsaStep(cfg if cfg is not None else chain_config())
        self.L = _lib()
        self.nstate = self.L.salsa_gb300_chain_state_size(self.step.h)
        if self.nstate <= 0:
            raise api.SalsaError(2, "the chain needs a level-4 handle")

    def _desc(self, thermo, nsub, dt, kappa, ssat):
        d = ChainDesc()
        d.ncell = int(kappa.numel())
        d.nsub, d.dt = int(nsub), float(dt)
        d.temp, d.press, d.rs, d.dn = (_p(thermo[k]) for k in ("temp", "press", "rs", "dn"))
        d.kappa, d.ssat = _p(kappa), _p(ssat)
        return d

    def _check(self, rc, what):
        if rc != SALSA_OK:
            raise api.SalsaError(rc, f"{what}: {ERROR_NAMES.get(rc, rc)}")

    def adjoint_bytes(self, ncell, nsub, dt, ckpt_every):
        """Device memory of a forward + adjoint pair beyond its arrays (C-ABI query)."""
        b = self.L.salsa_gb300_chain_adjoint_bytes(self.step.h, int(ncell), int(nsub), float(dt), int(ckpt_every))
        if b < 0:
            raise api.SalsaError(1, "salsa_gb300_chain_adjoint_bytes")
        return b

    def auto_ckpt_every(self, ncell, nsub, dt, budget=None, fraction=0.5):
        """Checkpoint spacing for a forward + adjoint pair: every step while that fits,
        otherwise the smallest spacing whose memory fits (each step past a checkpoint is
        recomputed once in the adjoint).  The budget defaults to `fraction` of the free
        device memory."""
        if budget is None:
            budget = fraction * torch.cuda.mem_get_info()[0]
        for k in range(1, nsub + 1):
            if self.adjoint_bytes(ncell, nsub, dt, k) <= budget:
                return k
        raise api.SalsaError(3, f"the chain's adjoint needs more than {budget / 2**30:.1f} GiB at any spacing")

    def forward(self, x0, thermo, kappa, ssat, nsub, dt, ckpt_every=1, keep_checkpoints=True):
        """Returns (xN, checkpoints or None).  ckpt_every=None chooses the spacing from
        the free device memory (auto_ckpt_every); the checkpoints tensor then has
        ceil(nsub / spacing) rows, and the spacing is `self.last_ckpt_every`."""
        ncell = kappa.numel()
        if ckpt_every is None:
            ckpt_every = self.auto_ckpt_every(ncell, nsub, dt)
        self.last_ckpt_every = ckpt_every
        xN = torch.empty_like(x0)
        ck = None
        if keep_checkpoints:
            nck = (nsub + ckpt_every - 1) // ckpt_every
            ck = torch.empty((nck, ncell, self.nstate), dtype=torch.float64, device=x0.device)
        d = self._desc(thermo, nsub, dt, kappa, ssat)
        torch.cuda.synchronize()
        rc = self.L.salsa_gb300_chain_forward(self.step.h, C.byref(d), _p(x0), _p(xN), _p(ck), int(ckpt_every), None)
        self._check(rc, "chain forward")
        return xN, ck

    def tlm(self, x0, thermo, kappa, ssat, nsub, dt, dx0=None, dkappa=None, dssat=None):
        xN = torch.empty_like(x0)
        dxN = torch.empty_like(x0)
        d = self._desc(thermo, nsub, dt, kappa, ssat)
        torch.cuda.synchronize()
        rc = self.L.salsa_gb300_chain_tlm(self.step.h, C.byref(d), _p(x0), _p(dx0), _p(dkappa), _p(dssat), _p(xN),
                                          _p(dxN), None)
        self._check(rc, "chain tlm")
        return xN, dxN

    def adjoint(self, ck, ckpt_every, thermo, kappa, ssat, nsub, dt, xbarN):
        if ckpt_every is None:
            ckpt_every = self.last_ckpt_every     # the spacing of the last forward's checkpoints
        xbar0 = torch.empty_like(xbarN)
        kbar = torch.empty_like(kappa)
        sbar = torch.empty_like(ssat)
        d = self._desc(thermo, nsub, dt, kappa, ssat)
        torch.cuda.synchronize()
        rc = self.L.salsa_gb300_chain_adjoint(self.step.h, C.byref(d), _p(ck), int(ckpt_every), _p(xbarN.contiguous()),
                                              _p(xbar0), _p(kbar), _p(sbar), None)
        self._check(rc, "chain adjoint")
        return xbar0, kbar, sbar

    def close(self):
        self.step.close()


class _ChainFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, kappa, ssat, chain, thermo, nsub, dt, ckpt_every):
        xN, ck = chain.forward(x0, thermo, kappa, ssat, nsub, dt, ckpt_every)
        ctx.chain, ctx.thermo, ctx.nsub, ctx.dt, ctx.every = chain, thermo, nsub, dt, chain.last_ckpt_every
        ctx.save_for_backward(ck, kappa, ssat)
        return xN

    @staticmethod
    def backward(ctx, gN):
        ck, kappa, ssat = ctx.saved_tensors
        x0b, kb, sb = ctx.chain.adjoint(ck, ctx.every, ctx.thermo, kappa, ssat, ctx.nsub, ctx.dt, gN)
        return x0b, kb, sb, None, None, None, None, None


def chain_apply(chain, x0, kappa, ssat, thermo, nsub, dt, ckpt_every=None):
    """xN = chain(x0; kappa, ssat) as a differentiable torch operation.  By default the
    checkpoint spacing follows the free device memory (SalsaChain.auto_ckpt_every):
    every step while the chain fits, recomputation between checkpoints once it
    outgrows the memory."""
    return _ChainFn.apply(x0, kappa, ssat, chain, thermo, nsub, dt, ckpt_every)


def interior_cells(inp, t):
    """(nb, nyp, nxp, nzp) field -> (nb, ncell) of its interior cells, z fastest."""
    v = t[..., 2:inp.nyp - 2, 2:inp.nxp - 2, 1:inp.nzp - 1]
    return v.reshape(v.shape[0], -1)


def pack_state(inp):
    """[ncell, nstate] chain state and the thermodynamic inputs from make_inputs fields."""
    f = inp.fields
    lay = inp.layout
    n = torch.cat([interior_cells(inp, f[k]) for k in ("naero", "ncloud", "nprecp")], 0)
    ms = []
    nw = lay.nwet
    for s in range(nw):
        for k, nb in (("maero", lay.nbins), ("mcloud", lay.ncld), ("mprecp", lay.nprc)):
            ms.append(interior_cells(inp, f[k])[s * nb:(s + 1) * nb])
    x = torch.cat([n] + ms, 0).t().contiguous()
    T = interior_cells(inp, f["temp"][None])[0].contiguous()
    p = interior_cells(inp, f["press"][None])[0].contiguous()
    rs = interior_cells(inp, f["rsl"][None])[0].contiguous()
    dn = interior_cells(inp, f["dn"][None])[0].contiguous()
    kappa = interior_cells(inp, f["kappa"][None])[0].contiguous()
    rv = interior_cells(inp, f["rp"][None])[0]
    ssat = (rv / rs - 1.0).contiguous()
    return x, {"temp": T, "press": p, "rs": rs, "dn": dn}, kappa, ssat
