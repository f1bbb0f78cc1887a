"""tennet_gb300: the DMRG sweep hot path of TenNetLib.jl on one GB300 (sm_103a).

The Python API mirrors TenNetLib's Julia API for this path (Julia's trailing ``!`` becomes
a trailing ``_``):

=============================  ==============================================================
Python                          TenNetLib (file:line)
=============================  ==============================================================
``StateEnvs(psi, H)``           ``StateEnvs(psi, H::MPO)``          src/mps/state_envs.jl:54-60
``StateEnvs.position_``         ``position!``                       src/mps/state_envs.jl:364-367
``StateEnvs.product``           ``product`` / ``sysenv(v)``         src/mps/state_envs.jl:376-380
``update_position_``            ``update_position!``                src/mps/update_site.jl:231-277
``fullsweep_``                  ``fullsweep!``                      src/mps/sweep.jl:94-196
``SweepData``                   ``SweepData``                       src/mps/sweep.jl:26-35
``DMRGParams``                  ``DMRGParams``                      src/mps/dmrg.jl:26-102
``dmrg_`` / ``dmrg`` / ``dmrg2`` ``dmrg!`` / ``dmrg`` / ``dmrg2``    src/mps/dmrg.jl:148-301
``eig_solver``                  ``eig_solver``                      src/base/solver.jl:23-43
``exp_solver``                  ``exp_solver``                      src/base/solver.jl:66-88
``TDVPEngine`` / ``tdvpsweep_``  ``TDVPEngine`` / ``tdvpsweep!``      src/mps/tdvp.jl:17-277
``entropy``                     ``_entropy``                        src/mps/measure.jl:4-20
``measure(psi, "Sz")``          ``measure``                         src/mps/measure.jl:150-219
``ttn.*``                       the TTN path (``TTN``, ``StateEnvsTTN``, ``optimize!``; see ttn.py)
=============================  ==============================================================

All arithmetic runs in libtennet_cuda.so; this module only moves host arrays across the C
ABI.  It refuses to run without the library or without a GB300.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import models  # noqa: F401
from . import ttn  # noqa: F401
from ._lib import TenNetError

FLOAT64_THRESHOLD = 1e-15
INT32_MAX = 2**31 - 1

__all__ = [
    "Context", "MPO", "MPS", "StateEnvs", "DMRGParams", "SweepData", "eig_solver",
    "update_position_", "fullsweep_", "dynamic_fullsweep_", "updateH_", "dmrg_", "dmrg", "dmrg2",
    "entropy", "svd_truncate",
    "Float64_threshold", "TenNetError", "models", "TDVPEngine", "tdvpsweep_", "exp_solver",
    "ttn", "measure",
]

_threshold = [FLOAT64_THRESHOLD]


def Float64_threshold(value: float | None = None) -> float:
    """``Float64_threshold()`` (src/base/global_variables.jl:19-26)."""
    if value is not None:
        _threshold[0] = float(value)
    return _threshold[0]


class Context:
    """One GB300, one stream and its memory pool."""

    _default = None

    def __init__(self, device: int = 0, precision: str = "fp64", slices: int = 5,
                 svd_split: int | None = None):
        self.lib = L.load()
        self._users = 0
        self._closing = False
        h = L.vp()
        L.check(self.lib.tn_ctx_create(device, C.byref(h)))
        self.h = h
        self.set_precision(precision, slices)
        if svd_split is not None:
            self.set_svd_split(svd_split)

    # Objects that own device handles of this context hold it; the context is destroyed
    # only after the last of them, whatever order the garbage collector finalises them in.
    def _hold(self):
        self._users += 1

    def _drop(self):
        self._users -= 1
        if self._closing and self._users <= 0:
            self._destroy()

    def _destroy(self):
        if getattr(self, "h", None):
            self.lib.tn_ctx_destroy(self.h)
            self.h = None

    def set_precision(self, precision: str, slices: int = 5):
        mode = {"fp64": L.TN_PREC_FP64, "split": L.TN_PREC_SPLIT}[precision]
        L.check(self.lib.tn_ctx_set_precision(self.h, mode, slices))
        self.precision = precision
        self.slices = slices

    def set_svd_split(self, ncols: int):
        """Charge blocks with more than ``ncols`` columns take the multi-SM block SVD (-1:
        the threshold is tuned per block-size histogram, the default)."""
        L.check(self.lib.tn_ctx_set_svd_split(self.h, int(ncols)))

    def svd_schedule(self) -> list:
        """The tuned block-SVD schedule: per 32-column bucket of a bond's largest block, the
        candidate thresholds (None: every block on one CTA), their measured milliseconds,
        whether the choice is settled, and the chosen threshold (None: one CTA each)."""
        n = C.c_int(0)
        L.check(self.lib.tn_ctx_svd_schedule(self.h, None, None, 0, C.byref(n)))
        cap = max(n.value, 1)
        ent = (C.c_int32 * (9 * cap))()
        ms = (C.c_float * (5 * cap))()
        L.check(self.lib.tn_ctx_svd_schedule(self.h, ent, ms, cap, C.byref(n)))
        big = 2147483647
        out = []
        for i in range(n.value):
            e = ent[9 * i: 9 * i + 9]
            k = e[1]
            th = [None if t == big else int(t) for t in e[4:4 + k]]
            out.append({"bucket": int(e[0]), "candidates": th,
                        "ms": [float(x) for x in ms[5 * i: 5 * i + k]],
                        "settled": e[2] != -1,
                        "chosen": None if e[2] in (-1, big) else int(e[2]),
                        "timed": int(e[3])})
        return out

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context()
        return cls._default

    def close(self):
        self._closing = True
        if self._users <= 0:
            self._destroy()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _own(obj, handle):
    """Record that obj owns a device handle of obj.ctx."""
    obj.h = handle
    obj.ctx._hold()


def _release(obj, destroy_name: str):
    """Destroy obj's device handle, then release its hold on the context."""
    h = getattr(obj, "h", None)
    if h:
        obj.h = None
        getattr(obj.ctx.lib, destroy_name)(h)
        obj.ctx._drop()


def _links_to_sectors(links):
    nsec, q, dim = [], [], []
    for lk in links:
        lk = np.asarray(lk)
        if lk.size and np.any(np.diff(lk) < 0):
            raise ValueError("link charges must be sorted ascending")
        ch, cnt = np.unique(lk, return_counts=True)
        nsec.append(len(ch))
        q += ch.tolist()
        dim += cnt.tolist()
    return nsec, q, dim


class MPO:
    """Device copy of an MPO given as dense site tensors W[i] (w_i, w_{i+1}, d, d)."""

    def __init__(self, W, delta, phys_q, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        self.N = len(W)
        self.d = len(phys_q)
        self.phys_q = np.asarray(phys_q, dtype=np.int32)
        self.W = [np.asarray(w, dtype=np.float64) for w in W]   # host copies (MPO sums)
        self.delta = [np.asarray(x, dtype=np.int32) for x in delta]
        wd = [W[0].shape[0]] + [w.shape[1] for w in W]
        flat = np.concatenate([np.asarray(w, dtype=np.float64).ravel(order="F") for w in W])
        q = np.concatenate([np.asarray(x, dtype=np.int32) for x in delta])
        a1, p1 = L.as_i32(self.phys_q)
        a2, p2 = L.as_i32(wd)
        a3, p3 = L.as_i32(q)
        a4, p4 = L.as_f64(flat)
        h = L.vp()
        L.check(self.ctx.lib.tn_mpo_create(self.ctx.h, self.N, self.d, p1, p2, p3, p4, C.byref(h)))
        _own(self, h)

    @classmethod
    def from_terms(cls, N, terms, conserve_qns=True, ctx=None):
        W, delta, pq = models.mpo_from_terms(N, terms, conserve_qns)
        return cls(W, delta, pq, ctx)

    @classmethod
    def sum(cls, mpos):
        """The Hamiltonian H_1 + H_2 + ... of ``StateEnvs(psi, Vector{MPO})`` (ProjMPOSum2,
        ``src/mps/projmposum2.jl``) as one MPO with block-diagonal bonds, whose H_eff products
        are the sums of the summands' products."""
        mpos = list(mpos)
        if not mpos:
            raise ValueError("no MPO to sum")
        ctx = mpos[0].ctx
        for m in mpos:
            if m.ctx is not ctx or not np.array_equal(m.phys_q, mpos[0].phys_q):
                raise ValueError("the MPOs of a sum need one context and the same sites")
        W, delta = models.mpo_direct_sum([(m.W, m.delta) for m in mpos])
        return cls(W, delta, mpos[0].phys_q, ctx)

    def __del__(self):
        try:
            _release(self, "tn_mpo_destroy")
        except Exception:
            pass


class MPS:
    """Device MPS.  Created from dense site tensors (Dl, d, Dr) and link charge arrays."""

    def __init__(self, tensors=None, links=None, phys_q=None, center: int = 0,
                 ctx: Context | None = None, _handle=None, _N=None, _d=None):
        self.ctx = ctx or Context.default()
        if _handle is not None:
            _own(self, _handle)
            self.N = _N
            self.d = _d
            self.phys_q = np.asarray(phys_q, dtype=np.int32)
            return
        self.N = len(tensors)
        self.d = len(phys_q)
        self.phys_q = np.asarray(phys_q, dtype=np.int32)
        nsec, q, dim = _links_to_sectors(links)
        cplx = any(np.iscomplexobj(t) for t in tensors)
        if cplx:  # interleaved (re, im): ComplexF64 memory
            flat = np.concatenate([np.asarray(t, dtype=np.complex128).ravel(order="F")
                                   for t in tensors]).view(np.float64)
        else:
            flat = np.concatenate([np.asarray(t, dtype=np.float64).ravel(order="F")
                                   for t in tensors])
        bufs = [L.as_i32(self.phys_q), L.as_i32(nsec), L.as_i32(q), L.as_i32(dim), L.as_f64(flat)]
        h = L.vp()
        create = self.ctx.lib.tn_mps_create_complex if cplx else self.ctx.lib.tn_mps_create
        L.check(create(self.ctx.h, self.N, self.d, bufs[0][1], bufs[1][1], bufs[2][1], bufs[3][1],
                       bufs[4][1], center, C.byref(h)))
        _own(self, h)

    @classmethod
    def from_blocks(cls, blocks, links, phys_q, center: int = 0, ctx: Context | None = None):
        """MPS from charge blocks only (``tn_mps_create_blocks``): ``blocks[i]`` is site i's
        data in the block order of the C ABI (left sectors by ascending charge, then physical
        states, each Dl x Dr block column-major, see ``dense_to_blocks``); ``links`` are the
        per-basis-state charge arrays of links 0..N."""
        ctx = ctx or Context.default()
        phys_q = np.asarray(phys_q, dtype=np.int32)
        N = len(blocks)
        nsec, q, dim = _links_to_sectors(links)
        flat = np.concatenate([np.asarray(b, dtype=np.float64).ravel() for b in blocks])
        lens = np.ascontiguousarray([np.asarray(b).size for b in blocks], dtype=np.int64)
        bufs = [L.as_i32(phys_q), L.as_i32(nsec), L.as_i32(q), L.as_i32(dim), L.as_f64(flat)]
        h = L.vp()
        L.check(ctx.lib.tn_mps_create_blocks(ctx.h, N, len(phys_q), bufs[0][1], bufs[1][1],
                                             bufs[2][1], bufs[3][1], bufs[4][1],
                                             lens.ctypes.data_as(C.POINTER(C.c_int64)),
                                             center, C.byref(h)))
        return cls(ctx=ctx, _handle=h, _N=N, _d=len(phys_q), phys_q=phys_q)

    def site_blocks(self, i):
        """Site i as charge blocks in the order of ``from_blocks`` (1-D array)."""
        n = C.c_int64()
        L.check(self.ctx.lib.tn_mps_site_blocks(self.h, i, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        L.check(self.ctx.lib.tn_mps_site_blocks(self.h, i, out.ctypes.data_as(L.f64p), out.size,
                                                C.byref(n)))
        return out

    @classmethod
    def product(cls, states, phys_q, ctx=None):
        t, lk = models.product_state(states, phys_q)
        return cls(t, lk, phys_q, 0, ctx)

    @classmethod
    def random_product(cls, N, d, seed, ctx=None):
        t, lk = models.random_product_state(N, d, seed)
        return cls(t, lk, np.zeros(d, dtype=np.int32), 0, ctx)

    def link(self, i):
        """(charges, dims) of link i (0..N)."""
        n = C.c_int32()
        L.check(self.ctx.lib.tn_mps_link(self.h, i, C.byref(n), None, None, 0))
        q = np.zeros(n.value, dtype=np.int32)
        dm = np.zeros(n.value, dtype=np.int32)
        L.check(self.ctx.lib.tn_mps_link(self.h, i, C.byref(n), q.ctypes.data_as(L.i32p),
                                         dm.ctypes.data_as(L.i32p), n.value))
        return q, dm

    def link_charges(self, i):
        q, dm = self.link(i)
        return np.repeat(q, dm)

    def linkdims(self):
        return [int(self.link(i)[1].sum()) for i in range(1, self.N)]

    def maxlinkdim(self):
        return max(self.linkdims())

    @property
    def is_complex(self) -> bool:
        return self.ctx.lib.tn_mps_is_complex(self.h) == 1

    def to_complex_(self):
        """Make the state complex in place (imaginary parts zero)."""
        L.check(self.ctx.lib.tn_mps_make_complex(self.h))
        return self

    def site(self, i):
        """Dense site tensor (Dl, d, Dr): float64, or complex128 for a complex state."""
        Dl = int(self.link(i)[1].sum())
        Dr = int(self.link(i + 1)[1].sum())
        if self.is_complex:
            out = np.zeros(2 * Dl * self.d * Dr)
            L.check(self.ctx.lib.tn_mps_site_complex(self.h, i, out.ctypes.data_as(L.f64p),
                                                     out.size))
            return out.view(np.complex128).reshape((Dl, self.d, Dr), order="F")
        out = np.zeros(Dl * self.d * Dr)
        L.check(self.ctx.lib.tn_mps_site(self.h, i, out.ctypes.data_as(L.f64p), out.size))
        return out.reshape((Dl, self.d, Dr), order="F")

    @property
    def center(self):
        return self.ctx.lib.tn_mps_center(self.h)

    def inner(self, other: "MPS"):
        """<self|other> (both states on this context, same sites); complex when either is."""
        if self.is_complex or other.is_complex:
            v = np.zeros(2)
            L.check(self.ctx.lib.tn_mps_overlap_complex(self.h, other.h,
                                                        v.ctypes.data_as(L.f64p)))
            return complex(v[0], v[1])
        v = C.c_double()
        L.check(self.ctx.lib.tn_mps_overlap(self.h, other.h, C.byref(v)))
        return v.value

    def expect_local(self, op):
        """<psi|O_i|psi> / <psi|psi> for every site i (op: d x d matrix [s', s])."""
        op = np.asarray(op, dtype=np.float64)
        if op.shape != (self.d, self.d):
            raise ValueError("operator must be d x d")
        flat = np.ascontiguousarray(op.ravel(order="F"))
        out = np.zeros(self.N)
        L.check(self.ctx.lib.tn_mps_expect_local(self.h, flat.ctypes.data_as(L.f64p),
                                                 out.ctypes.data_as(L.f64p)))
        return out

    def __len__(self):
        return self.N

    def __del__(self):
        try:
            _release(self, "tn_mps_destroy")
        except Exception:
            pass


class StateEnvs:
    """``StateEnvs(psi, H::MPO)``: a copy of psi plus lazily built ProjMPO environments.

    ``StateEnvs(psi, H, Ms, weight=w)`` (``src/mps/state_envs.jl:88-105``) adds the
    excited-state projectors of the states Ms: the effective Hamiltonian becomes
    ProjMPO_MPS2's, H_eff + w sum_k |m_k><m_k| (``src/mps/projmpo_mps2.jl:94-101``).
    ``StateEnvs(psi, [H1, H2, ...])`` (``state_envs.jl:70-78``, ProjMPOSum2) takes the sum of
    the MPOs through ``MPO.sum``."""

    def __init__(self, psi: MPS, H: MPO, Ms=None, *, weight=None):
        self.ctx = psi.ctx
        if isinstance(H, (list, tuple)):  # StateEnvs(psi, Vector{MPO}): ProjMPOSum2
            H = MPO.sum(H)
        self.H = H
        self.phys_q = psi.phys_q
        self.N = psi.N
        self.d = psi.d
        h = L.vp()
        L.check(self.ctx.lib.tn_env_create(psi.h, H.h, C.byref(h)))
        _own(self, h)
        self._nproj = 0
        if Ms is not None:
            self.set_projectors(Ms, weight)

    def set_projectors(self, Ms, weight):
        """Excited-state projectors (copies of the states in Ms) with the given weight."""
        Ms = list(Ms)
        arr = (L.vp * max(len(Ms), 1))(*[m.h for m in Ms])
        w = -1.0 if weight is None else float(weight)
        L.check(self.ctx.lib.tn_env_set_projectors(self.h, arr, len(Ms), w))
        self._nproj = len(Ms)
        return self

    def bond_spectra(self):
        """The kept spectrum of every bond from the last full sweep (``SweepData.lasteigs``):
        N - 1 arrays of descending squared singular values, empty before the first sweep."""
        counts = np.zeros(max(self.N - 1, 1), dtype=np.int32)
        lib = self.ctx.lib
        L.check(lib.tn_env_bond_spectra(self.h, None, 0, counts.ctypes.data_as(L.i32p),
                                        len(counts)))
        out = np.zeros(max(int(counts.sum()), 1))
        L.check(lib.tn_env_bond_spectra(self.h, out.ctypes.data_as(L.f64p), len(out),
                                        counts.ctypes.data_as(L.i32p), len(counts)))
        offs = np.concatenate([[0], np.cumsum(counts[: self.N - 1])])
        return [out[offs[b]:offs[b + 1]].copy() for b in range(self.N - 1)]

    def __len__(self):
        return self.N

    @property
    def psi(self) -> MPS:
        return self.getpsi()

    def getpsi(self) -> MPS:
        h = L.vp()
        L.check(self.ctx.lib.tn_env_getpsi(self.h, C.byref(h)))
        return MPS(ctx=self.ctx, _handle=h, _N=self.N, _d=self.d, phys_q=self.phys_q)

    def position_(self, pos: int, nsite: int = 2):
        """``position!`` + ``set_nsite!`` (0-based pos)."""
        L.check(self.ctx.lib.tn_env_position(self.h, pos, nsite))
        self._pos = pos
        return self

    def product(self, v):
        """H_eff * v at the current position, v dense (Dl, d, d, Dr); complex for a complex
        state."""
        if np.iscomplexobj(v) or self.is_complex:
            v = np.asarray(v, dtype=np.complex128)
            flat = np.ascontiguousarray(v.ravel(order="F"))
            out = np.zeros_like(flat)
            L.check(self.ctx.lib.tn_env_product_complex(
                self.h, flat.view(np.float64).ctypes.data_as(L.f64p),
                out.view(np.float64).ctypes.data_as(L.f64p), flat.size))
            return out.reshape(v.shape, order="F")
        v = np.asarray(v, dtype=np.float64)
        flat = np.ascontiguousarray(v.ravel(order="F"))
        out = np.zeros_like(flat)
        L.check(self.ctx.lib.tn_env_product(self.h, flat.ctypes.data_as(L.f64p),
                                            out.ctypes.data_as(L.f64p), flat.size))
        return out.reshape(v.shape, order="F")

    @property
    def is_complex(self) -> bool:
        h = L.vp()
        L.check(self.ctx.lib.tn_env_getpsi(self.h, C.byref(h)))
        try:
            return self.ctx.lib.tn_mps_is_complex(h) == 1
        finally:
            self.ctx.lib.tn_mps_destroy(h)

    def to_complex_(self):
        """Make the state and its environments complex (imaginary parts zero)."""
        L.check(self.ctx.lib.tn_env_make_complex(self.h))
        return self

    __call__ = product

    def environment(self, side: str, i: int):
        """Dense environment L[i] ("left") or R[i] ("right") as [bra, MPO state, ket]."""
        sd = {"left": 0, "right": 1}[side]
        dims = np.zeros(3, dtype=np.int32)
        L.check(self.ctx.lib.tn_env_environment(self.h, sd, i, None, 0,
                                                dims.ctypes.data_as(L.i32p)))
        out = np.zeros(int(np.prod(dims.astype(np.int64))))
        L.check(self.ctx.lib.tn_env_environment(self.h, sd, i, out.ctypes.data_as(L.f64p),
                                                out.size, dims.ctypes.data_as(L.i32p)))
        return out.reshape(tuple(int(x) for x in dims), order="F")

    def product_flops(self) -> float:
        f = C.c_double()
        L.check(self.ctx.lib.tn_env_product_flops(self.h, C.byref(f)))
        return f.value

    def __del__(self):
        try:
            _release(self, "tn_env_destroy")
        except Exception:
            pass


SPIN_HALF_OPS = {
    "Sz": np.diag([0.5, -0.5]),
    "Sx": np.array([[0.0, 0.5], [0.5, 0.0]]),
    "S+": np.array([[0.0, 1.0], [0.0, 0.0]]),
    "S-": np.array([[0.0, 0.0], [1.0, 0.0]]),
    "Id": np.eye(2),
    "Nup": np.diag([1.0, 0.0]),
    "Ndn": np.diag([0.0, 1.0]),
}


def dense_to_blocks(t, ql, phys_q, qr):
    """Charge blocks of a dense site tensor t[l, s, r] in the order of the C ABI's
    ``tn_mps_create_blocks``: left sectors by ascending charge, then physical states, each
    Dl x Dr block column-major."""
    t = np.asarray(t, dtype=np.float64)
    ql, qr = np.asarray(ql), np.asarray(qr)
    out = []
    for a in np.unique(ql):
        rows = np.nonzero(ql == a)[0]
        for s, qs in enumerate(np.asarray(phys_q)):
            cols = np.nonzero(qr == a + qs)[0]
            if len(cols):
                out.append(t[np.ix_(rows, [s], cols)][:, 0, :].ravel(order="F"))
    return np.concatenate(out) if out else np.zeros(0)


def blocks_to_dense(b, ql, phys_q, qr):
    """Inverse of ``dense_to_blocks``: the dense site tensor (Dl, d, Dr)."""
    ql, qr = np.asarray(ql), np.asarray(qr)
    pq = np.asarray(phys_q)
    t = np.zeros((len(ql), len(pq), len(qr)))
    off = 0
    for a in np.unique(ql):
        rows = np.nonzero(ql == a)[0]
        for s, qs in enumerate(pq):
            cols = np.nonzero(qr == a + qs)[0]
            if len(cols):
                n = len(rows) * len(cols)
                t[np.ix_(rows, [s], cols)] = np.asarray(b[off:off + n]).reshape(
                    (len(rows), len(cols)), order="F")[:, None, :]
                off += n
    return t

def measure(psi: MPS, op, pos: int | None = None, sites=None):
    """``measure(Float64, psi, opstr[, pos]; sites)`` (``src/mps/measure.jl:150-219``):
    local expectation values of a single-site operator, given by S=1/2 name ("Sz", "Sx",
    "S+", "S-", "Id", "Nup", "Ndn") or as a d x d matrix [s', s].  pos (0-based) returns one
    value; sites selects a subset; default all sites.

    With a list of (operator, site) pairs, ``measure(T, psi, ["Sz" => i, "Sz" => j, ...])``
    (src/mps/measure.jl:222-330, bosonic): <psi| O_i O_j ... |psi> / <psi|psi> (operators on
    one site multiplied in order).  Each operator is split into its parts of definite charge
    change q(s') - q(s); every combination whose changes add to zero is an MPO of bond
    dimension one (link charges the running sum of the changes), evaluated on the GPU as
    <phi| H_eff |phi> of the two-site tensor phi at the orthogonality centre, between the
    environments of that MPO; the other combinations vanish in a state of definite charge."""
    if isinstance(op, (list, tuple)) and op and isinstance(op[0], (list, tuple)):
        return _measure_product(psi, op)
    mat = SPIN_HALF_OPS[op] if isinstance(op, str) else np.asarray(op, dtype=np.float64)
    vals = psi.expect_local(mat)
    if pos is not None:
        return float(vals[pos])
    if sites is not None:
        return [float(vals[i]) for i in sites]
    return [float(v) for v in vals]


def _measure_product(psi: MPS, oppairs):
    import itertools
    d, pq = psi.d, np.asarray(psi.phys_q)
    ops = {}
    for name, site in oppairs:
        m = SPIN_HALF_OPS[name] if isinstance(name, str) else np.asarray(name, dtype=np.float64)
        if m.shape != (d, d):
            raise ValueError("an operator must be a d x d matrix [s', s]")
        site = int(site)
        ops[site] = ops[site] @ m if site in ops else m
    sites = sorted(ops)
    parts = []
    for site in sites:
        comp = {}
        for sp in range(d):
            for s0 in range(d):
                if ops[site][sp, s0] != 0.0:
                    comp.setdefault(int(pq[sp] - pq[s0]), np.zeros((d, d)))[sp, s0] = ops[site][sp, s0]
        parts.append(sorted(comp.items()) or [(0, np.zeros((d, d)))])
    N, c = psi.N, psi.center
    pos = min(c, N - 2)  # the two-site window [pos, pos + 1] holds the centre
    phi = np.tensordot(psi.site(pos), psi.site(pos + 1), axes=([2], [0]))
    eye = np.eye(d)
    total = 0.0
    for combo in itertools.product(*parts):
        if sum(dq for dq, _ in combo) != 0:
            continue
        which = dict(zip(sites, combo))
        W, delta, q = [], [np.zeros(1, dtype=np.int32)], 0
        for i in range(N):
            dq, m = which.get(i, (0, eye))
            W.append(np.asarray(m, dtype=np.float64).reshape(1, 1, d, d))
            q += dq
            delta.append(np.array([q], dtype=np.int32))
        env = StateEnvs(psi, MPO(W, delta, pq, psi.ctx))
        env.position_(pos, 2)
        total = total + np.vdot(phi, env.product(phi))
    nrm = psi.inner(psi)
    val = total / nrm
    return complex(val) if np.iscomplexobj(val) and abs(np.imag(val)) > 1e-13 else float(np.real(val))


def exp_solver(*_args, **_kwargs):
    """Token for the Krylov exponential solver (``src/base/solver.jl:66-88``); the solve
    runs inside libtennet_cuda.so as part of each TDVP update step."""
    raise TypeError("exp_solver is passed to tdvpsweep_, not called")


def eig_solver(*_args, **_kwargs):
    """Token for the Lanczos ground-state solver (``src/base/solver.jl:23-43``).  The solve
    itself runs inside libtennet_cuda.so as part of each update step."""
    raise TypeError("eig_solver is passed to update_position_/fullsweep_, not called")


def _params(kwargs, exp=False) -> L.UpdateParams:
    p = L.UpdateParams()
    maxdim = kwargs.get("maxdim", INT32_MAX)
    p.maxdim = int(min(maxdim, INT32_MAX))
    p.mindim = int(kwargs.get("mindim", 1))
    p.cutoff = float(kwargs.get("cutoff", Float64_threshold()))
    p.normalize = int(bool(kwargs.get("normalize", True)))
    p.krylovdim = int(kwargs.get("solver_krylovdim", 30 if exp else 5))
    p.maxiter = int(kwargs.get("solver_maxiter", 100 if exp else 2))
    p.tol = float(kwargs.get("solver_tol", 1e-12 if exp else 1e-14))
    p.eager = int(bool(kwargs.get("solver_eager", exp)))
    p.check_convergence = int(bool(kwargs.get("solver_check_convergence", False)))
    p.noise = float(kwargs.get("noise", 0.0))
    if not kwargs.get("ishermitian", True):
        raise ValueError("only Hermitian effective Hamiltonians are built")
    if kwargs.get("time_step") is not None and not exp:
        raise ValueError("time evolution goes through tdvpsweep_")
    return p


def update_position_(sysenv: StateEnvs, solver, pos: int, nsite: int, ortho: str, **kwargs):
    """``update_position!`` for one- or two-site DMRG (``src/mps/update_site.jl:231-277``).
    Returns (energy, truncerr, eigs)."""
    if solver is not eig_solver:
        raise ValueError("only eig_solver is built")
    if nsite not in (1, 2):
        raise ValueError("nsite must be 1 or 2")
    p = _params(kwargs)
    res = L.UpdateResult()
    cap = max(int(p.maxdim if p.maxdim < 1 << 20 else 1 << 16), 1)
    eigs = np.zeros(cap)
    o = {"left": L.TN_ORTHO_LEFT, "right": L.TN_ORTHO_RIGHT}[ortho]
    L.check(sysenv.ctx.lib.tn_env_update_position_nsite(sysenv.h, pos, nsite, o, C.byref(p),
                                                        C.byref(res),
                                                        eigs.ctypes.data_as(L.f64p), cap))
    return res.energy, res.truncerr, eigs[: res.neigs].copy()


@dataclass
class SweepData:
    """History of full sweeps (``src/mps/sweep.jl:26-35``)."""

    sweepcount: int = 0
    maxchi: list = field(default_factory=list)
    energy: list = field(default_factory=list)
    entropy: list = field(default_factory=list)
    maxtruncerr: list = field(default_factory=list)
    lasteigs: list = field(default_factory=list)
    # per-sweep device timings and work (not in the reference; from CUDA events)
    stats: list = field(default_factory=list)


def entropy(p) -> float:
    """von Neumann entropy -sum p log p (``src/mps/measure.jl:4-20``)."""
    p = np.asarray(p, dtype=np.float64)
    s = float(p.sum())
    if abs(s - 1.0) > 100 * Float64_threshold():
        p = p / s
    return float(-sum(a * math.log(a) for a in p if a > 0.0))


def fullsweep_(sysenv: StateEnvs, solver, nsite: int, swdata: SweepData, **kwargs):
    """``fullsweep!``: left-to-right then right-to-left one- or two-site updates
    (``src/mps/sweep.jl:94-196``).

    Returns (Delta E, Delta S) and appends to ``swdata``.
    """
    if solver is not eig_solver or nsite not in (1, 2):
        raise ValueError("only one- and two-site eig_solver sweeps are built")
    p = _params(kwargs)
    outputlevel = kwargs.get("outputlevel", 1)
    res = L.SweepResult()
    cap = max(int(p.maxdim if p.maxdim < 1 << 20 else 1 << 16), 1)
    mid = np.zeros(cap)
    nmid = C.c_int32()
    swdata.sweepcount += 1
    t0 = time.perf_counter()
    L.check(sysenv.ctx.lib.tn_env_fullsweep_nsite(sysenv.h, nsite, C.byref(p), C.byref(res),
                                                  mid.ctypes.data_as(L.f64p), cap,
                                                  C.byref(nmid)))
    wall = time.perf_counter() - t0
    mid = mid[: nmid.value].copy()
    swdata.maxchi.append(int(res.maxlinkdim))
    swdata.energy.append(float(res.energy))
    swdata.entropy.append(entropy(mid / mid.sum()) if mid.size else 0.0)
    swdata.maxtruncerr.append(float(res.maxtruncerr))
    swdata.lasteigs = sysenv.bond_spectra()
    swdata.stats.append({
        "matvecs": res.matvecs, "heff_flops": res.heff_flops, "heff_ms": res.heff_ms,
        "env_ms": res.env_ms, "svd_ms": res.svd_ms, "lanczos_ms": res.lanczos_ms,
        "sweep_ms": res.sweep_ms, "gemm_ms": res.gemm_ms, "gemm_flops": res.gemm_flops, "pack_ms": res.pack_ms,
        "gemm_launches": res.gemm_launches, "kernel_launches": res.kernel_launches,
        "krylov_bytes": res.krylov_bytes, "svd_gemm_flops": res.svd_gemm_flops,
        "svd_jacobi_flops": res.svd_jacobi_flops, "svd_sweeps32": res.svd_sweeps32,
        "svd_sweeps_df": res.svd_sweeps_df, "svd_small_flops": res.svd_small_flops,
        "wall_s": wall})
    if swdata.sweepcount > 1:
        enerr = swdata.energy[-1] - swdata.energy[-2]
        enterr = swdata.entropy[-1] - swdata.entropy[-2]
    else:
        enerr = enterr = float("nan")
    if outputlevel > 0:
        print("-" * 83)
        print(f"At sweep {swdata.sweepcount} => E={swdata.energy[-1]}, S={swdata.entropy[-1]}, "
              f"MaxLinkDim={swdata.maxchi[-1]}, Noise={p.noise:.2g}")
        print(f"At sweep {swdata.sweepcount} => ΔE={enerr}, ΔS={enterr}, "
              f"MaxErr={swdata.maxtruncerr[-1]:.2g}, Time={round(wall, 3)}")
        print("-" * 83)
    return enerr, enterr


def _record_sweep(swdata, res, mid, wall, spectra):
    mid = np.asarray(mid)
    swdata.sweepcount += 1
    swdata.maxchi.append(int(res.maxlinkdim))
    swdata.energy.append(float(res.energy))
    swdata.entropy.append(entropy(mid / mid.sum()) if mid.size else 0.0)
    swdata.maxtruncerr.append(float(res.maxtruncerr))
    swdata.lasteigs = spectra
    swdata.stats.append({
        "matvecs": res.matvecs, "heff_flops": res.heff_flops, "heff_ms": res.heff_ms,
        "env_ms": res.env_ms, "svd_ms": res.svd_ms, "lanczos_ms": res.lanczos_ms,
        "sweep_ms": res.sweep_ms, "gemm_ms": res.gemm_ms, "gemm_flops": res.gemm_flops,
        "pack_ms": res.pack_ms, "gemm_launches": res.gemm_launches,
        "kernel_launches": res.kernel_launches, "krylov_bytes": res.krylov_bytes,
        "svd_gemm_flops": res.svd_gemm_flops, "svd_jacobi_flops": res.svd_jacobi_flops,
        "svd_sweeps32": res.svd_sweeps32, "svd_sweeps_df": res.svd_sweeps_df,
        "svd_small_flops": res.svd_small_flops, "wall_s": wall})


class TDVPEngine:
    """``TDVPEngine(psi, H)`` (``src/mps/tdvp.jl:17-64``): environments, sweep history and
    the absolute elapsed time of a TDVP run."""

    def __init__(self, psi: MPS, H: MPO):
        self.sysenv = StateEnvs(psi, H)
        self.swdata = SweepData()
        self.abstime = 0.0

    def getpsi(self) -> MPS:
        return self.sysenv.getpsi()

    def sweepcount(self):
        return self.swdata.sweepcount

    def getenergy(self):
        return self.swdata.energy[-1]

    def getentropy(self):
        return self.swdata.entropy[-1]

    def maxchi(self):
        return self.swdata.maxchi[-1]

    def totalerror(self):
        return float(sum(self.swdata.maxtruncerr))

    def sweeperror(self):
        return self.swdata.maxtruncerr[-1]

    def sweepdata(self):
        return self.swdata


def updateH_(target, H: MPO, Ms=None, *, weight=None, recalcEnv=True):
    """``updateH!`` of a ``StateEnvs`` (``src/mps/state_envs.jl:181-212, 241-260``) or of a
    ``TDVPEngine`` (``src/mps/tdvp.jl:182-196``): H replaces the Hamiltonian.  With
    ``recalcEnv`` every environment is rebuilt from H as positions are taken; without it (a
    single MPO only, after a full sweep, same MPO link indices) the environments built so far
    stay, so the next half sweep reads right environments of the old H, as in the reference.
    A StateEnvs with excited-state projectors takes the new states ``Ms`` and ``weight`` too
    (``recalcEnv`` true only)."""
    sysenv = target.sysenv if isinstance(target, TDVPEngine) else target
    if isinstance(H, (list, tuple)):
        if not recalcEnv:
            raise ValueError(f"`updateH!()` :: Not implemented for `recalcEnv={recalcEnv}` "
                             "with `ProjMPOSum2` !!")
        H = MPO.sum(H)
    if Ms is not None and not sysenv._nproj:
        raise ValueError("`updateH!()` with Ms needs a StateEnvs made with projector states")
    if sysenv._nproj and Ms is None:
        raise ValueError("`updateH!()` of a StateEnvs with projector states takes Ms and weight")
    if sysenv._nproj and not recalcEnv:
        raise ValueError(f"`updateH!()` :: Not implemented for `recalcEnv={recalcEnv}` with "
                         "excited-state projectors !!")
    if H.ctx is not sysenv.ctx:
        raise ValueError("the MPO belongs to another context")
    L.check(sysenv.ctx.lib.tn_env_update_mpo(sysenv.h, H.h, int(bool(recalcEnv))))
    sysenv.H = H
    if Ms is not None:
        sysenv.set_projectors(Ms, weight)
    return None


def _sweep_printout(swdata, wall, noise, outputlevel):
    if swdata.sweepcount > 1 and len(swdata.energy) > 1:
        enerr = swdata.energy[-1] - swdata.energy[-2]
        enterr = swdata.entropy[-1] - swdata.entropy[-2]
    else:
        enerr = enterr = float("nan")
    if outputlevel > 0:
        print("-" * 83)
        print(f"At sweep {swdata.sweepcount} => E={swdata.energy[-1]}, S={swdata.entropy[-1]}, "
              f"MaxLinkDim={swdata.maxchi[-1]}, Noise={noise:.2g}")
        print(f"At sweep {swdata.sweepcount} => ΔE={enerr}, ΔS={enterr}, "
              f"MaxErr={swdata.maxtruncerr[-1]:.2g}, Time={round(wall, 3)}")
        print("-" * 83)
    return enerr, enterr


def _dynamic_sweep(sysenv, swdata, tau, eigthreshold, **kwargs):
    """The mixed one-/two-site sweep of ``dynamic_fullsweep!`` (``src/mps/sweep.jl:284-355``)
    with the eigensolver (tau None) or the exponential solver at tau/2 per update.  Returns the
    per-bond choices (left half, right half)."""
    N = sysenv.N
    if len(swdata.lasteigs) != N - 1 or any(len(e) == 0 for e in swdata.lasteigs):
        raise ValueError("dynamic_fullsweep!: swdata.lasteigs must hold the spectra of the "
                         f"{N - 1} bonds from a previous full sweep of this state")
    last_min = np.array([float(np.asarray(e)[-1]) for e in swdata.lasteigs], dtype=np.float64)
    choices = np.zeros(2 * (N - 1), dtype=np.int32)
    p = _params(kwargs, exp=tau is not None)
    res = L.SweepResult()
    cap = max(int(p.maxdim if p.maxdim < 1 << 20 else 1 << 16), 1)
    mid = np.zeros(cap)
    nmid = C.c_int32()
    lib = sysenv.ctx.lib
    t0 = time.perf_counter()
    if tau is None:
        L.check(lib.tn_env_fullsweep_dynamic(
            sysenv.h, float(eigthreshold), last_min.ctypes.data_as(L.f64p),
            choices.ctypes.data_as(L.i32p), C.byref(p), C.byref(res),
            mid.ctypes.data_as(L.f64p), cap, C.byref(nmid)))
    else:
        tau = complex(tau)
        L.check(lib.tn_env_tdvpsweep_dynamic(
            sysenv.h, tau.real, tau.imag, float(eigthreshold), last_min.ctypes.data_as(L.f64p),
            choices.ctypes.data_as(L.i32p), C.byref(p), C.byref(res),
            mid.ctypes.data_as(L.f64p), cap, C.byref(nmid)))
    wall = time.perf_counter() - t0
    _record_sweep(swdata, res, mid[: nmid.value], wall, sysenv.bond_spectra())
    left, right = choices[: N - 1].copy(), choices[N - 1:].copy()
    swdata.stats[-1]["nsite_left"], swdata.stats[-1]["nsite_right"] = left, right
    _sweep_printout(swdata, wall, p.noise, kwargs.get("outputlevel", 1))
    return left, right


def _needs_extension(sysenv, swdata, extendat):
    """``dynamic_fullsweep!``'s first sweep and every extendat-th sweep (``sweep.jl:
    266-282``): global subspace expansion then a one-site sweep for a single MPO, a two-site
    sweep when excited-state projectors are present."""
    ext = swdata.sweepcount == 0 or (extendat is not None
                                     and (swdata.sweepcount + 1) % int(extendat) == 0)
    if ext and not sysenv._nproj:
        raise NotImplementedError(
            "dynamic_fullsweep!: this sweep of a single-MPO StateEnvs starts with krylov_extend! "
            "(global subspace expansion), which is not built; run a sweep with a fixed nsite "
            "first (and leave extendat = nothing)")
    return ext


def dynamic_fullsweep_(sysenv: StateEnvs, solver, swdata: SweepData, eigthreshold=1e-12,
                       extendat=None, **kwargs):
    """``dynamic_fullsweep!`` (``src/mps/sweep.jl:257-355``): per bond a one-site update when
    the bond's last kept spectrum ends below ``eigthreshold`` or its link is at ``maxdim``,
    else a two-site update.  With ``exp_solver`` the keyword ``time_step`` is the step of each
    update (``tdvpsweep!`` passes half its step) and ``reverse_step`` must be true.  The
    sweeps that the reference opens with ``krylov_extend!`` raise ``NotImplementedError``
    (single MPO); with excited-state projectors they are two-site sweeps.  Returns
    (Delta E, Delta S)."""
    if solver is exp_solver:
        if kwargs.get("time_step") is None or not kwargs.get("reverse_step", False):
            raise ValueError("exp_solver sweeps need time_step and reverse_step = true")
        tau = 2.0 * complex(kwargs.pop("time_step"))
        kwargs.pop("reverse_step")
        if tau.imag == 0.0:
            tau = tau.real
    elif solver is eig_solver:
        tau = None
    else:
        raise ValueError("only eig_solver and exp_solver are built")
    if _needs_extension(sysenv, swdata, extendat):
        if tau is not None:
            raise ValueError("excited-state projectors are built for the eigensolver only")
        return fullsweep_(sysenv, solver, 2, swdata, **kwargs)
    _dynamic_sweep(sysenv, swdata, tau, eigthreshold, **kwargs)
    if swdata.sweepcount > 1 and len(swdata.energy) > 1:
        return (swdata.energy[-1] - swdata.energy[-2], swdata.entropy[-1] - swdata.entropy[-2])
    return float("nan"), float("nan")


def tdvpsweep_(engine: TDVPEngine, time_step, nsite=2, solver=exp_solver, **kwargs):
    """``tdvpsweep!`` (``src/mps/tdvp.jl:247-277``) with nsite = 2: one full sweep with
    ``exp_solver`` at time_step/2 and reverse one-site steps; ``abstime += |time_step|``.

    A real time step is imaginary-time evolution exp(time_step H); a complex one (real-time
    evolution exp(-i dt H) is ``time_step = -1j * dt``) makes the state complex first, as
    ITensors promotes the MPS to ComplexF64.  nsite = 1 is the one-site sweep with the
    zero-site reverse step.  ``nsite = "dynamic"`` is ``dynamic_fullsweep!``'s mixed sweep
    (keywords ``eigthreshold``, default 1e-12, and ``extendat``); its sweeps that open with
    global subspace expansion (the first one, every extendat-th) are not built and raise
    ``NotImplementedError``, so a dynamic run starts after one sweep with a fixed nsite.  The
    default nsite is 2 (the reference's default is "dynamic").
    """
    if solver is not exp_solver:
        raise ValueError("`tdvpsweep!()`: `solver` must be `exp_solver` !!")
    if nsite == "dynamic":
        if kwargs.get("noise", 0.0):
            raise ValueError("`updatePosition()` :: `noise` cannot be greater than zero for "
                             "`reverse_step=true` !!")
        eigthreshold = kwargs.pop("eigthreshold", 1e-12)
        extendat = kwargs.pop("extendat", None)
        _needs_extension(engine.sysenv, engine.swdata, extendat)
        _dynamic_sweep(engine.sysenv, engine.swdata, time_step, eigthreshold,
                       **{"outputlevel": 0, **kwargs})
        engine.abstime += abs(time_step)
        return None
    if nsite not in (1, 2):
        raise ValueError("`tdvpsweep!()`: `nsite` must be `\"dynamic\"`, `2`, or `1` !!")
    if kwargs.get("extendat") is not None:
        raise ValueError("`tdvpsweep!()`: `extendat` must be `nothing` for `nsite == 2` or "
                         "`nsite == 1`.")
    if kwargs.get("noise", 0.0):
        raise ValueError("`updatePosition()` :: `noise` cannot be greater than zero for "
                         "`reverse_step=true` !!")
    p = _params(kwargs, exp=True)
    res = L.SweepResult()
    cap = max(int(p.maxdim if p.maxdim < 1 << 20 else 1 << 16), 1)
    mid = np.zeros(cap)
    nmid = C.c_int32()
    sysenv = engine.sysenv
    t0 = time.perf_counter()
    tau = complex(time_step)
    if nsite == 1:
        L.check(sysenv.ctx.lib.tn_env_tdvpsweep_nsite(
            sysenv.h, 1, tau.real, tau.imag, C.byref(p), C.byref(res),
            mid.ctypes.data_as(L.f64p), cap, C.byref(nmid)))
    elif tau.imag != 0.0:
        L.check(sysenv.ctx.lib.tn_env_tdvpsweep_complex(
            sysenv.h, tau.real, tau.imag, C.byref(p), C.byref(res), mid.ctypes.data_as(L.f64p),
            cap, C.byref(nmid)))
    else:
        L.check(sysenv.ctx.lib.tn_env_tdvpsweep(sysenv.h, tau.real, C.byref(p), C.byref(res),
                                                mid.ctypes.data_as(L.f64p), cap, C.byref(nmid)))
    _record_sweep(engine.swdata, res, mid[: nmid.value], time.perf_counter() - t0,
                  sysenv.bond_spectra())
    engine.abstime += abs(time_step)
    return None


@dataclass
class DMRGParams:
    """Stage schedule of DMRG (``src/mps/dmrg.jl:26-102``)."""

    maxdim: list
    nsweeps: list
    cutoff: object = None
    noise: object = 0.0
    noisedecay: object = 1.0
    disable_noise_after: object = -1

    def __post_init__(self):
        n = len(self.nsweeps)
        if self.cutoff is None:
            self.cutoff = Float64_threshold()

        def vec(x, typ):
            return [typ(v) for v in x] if isinstance(x, (list, tuple, np.ndarray)) else [typ(x)] * n

        self.cutoff = vec(self.cutoff, float)
        self.noise = vec(self.noise, float)
        self.noisedecay = vec(self.noisedecay, float)
        self.disable_noise_after = vec(self.disable_noise_after, int)
        self.maxdim = [int(v) for v in self.maxdim]
        self.nsweeps = [int(v) for v in self.nsweeps]
        if not (len(self.maxdim) == n == len(self.cutoff) == len(self.noise) ==
                len(self.noisedecay) == len(self.disable_noise_after)):
            raise ValueError("`DMRGParams()` :: Size mismatch in input vectors !!")


def dmrg_(sysenv: StateEnvs, params: DMRGParams, nsite: int, **kwargs) -> SweepData:
    """``dmrg!`` stage loop (``src/mps/dmrg.jl:148-227``)."""
    outputlevel = kwargs.get("outputlevel", 1)
    enerrgoal = kwargs.get("energyErrGoal")
    enterrgoal = kwargs.get("entropyErrGoal")
    sw = SweepData()
    for ii in range(len(params.nsweeps)):
        noise = params.noise[ii]
        if outputlevel > 0:
            print("-" * 83)
            print(f"DMRG level={ii + 1} => maxdim={params.maxdim[ii]}, "
                  f"nsweeps={params.nsweeps[ii]}, cutoff={params.cutoff[ii]:.2E}")
            print("-" * 83)
        for jj in range(1, params.nsweeps[ii] + 1):
            kw = dict(kwargs)
            kw.update(maxdim=params.maxdim[ii], cutoff=params.cutoff[ii], noise=noise)
            enerr, enterr = fullsweep_(sysenv, eig_solver, nsite, sw, **kw)
            met = False
            if enerrgoal is not None and enterrgoal is not None:
                met = abs(enerr) < abs(enerrgoal) and abs(enterr) < abs(enterrgoal)
            elif enerrgoal is not None:
                met = abs(enerr) < abs(enerrgoal)
            # the reference's entropy-only branch discards its comparison
            # (src/mps/dmrg.jl:190-191), so it never stops early: kept as is.
            if met and abs(noise) < Float64_threshold():
                break
            if jj == params.disable_noise_after[ii]:
                noise = 0.0
            noise /= params.noisedecay[ii]
            if noise < 100 * Float64_threshold():
                noise = 0.0
    return sw


def dmrg(psi0: MPS, H: MPO, *args, **kwargs):
    """``dmrg(psi0, H, params, nsite)`` -> (energy, psi) (``src/mps/dmrg.jl:231-236``), or
    ``dmrg(psi0, H, Ms, params, nsite; weight)`` for the lowest state with the states Ms
    projected out (``src/mps/dmrg.jl:238-249``; weight must be > 0)."""
    if args and isinstance(args[0], (list, tuple)):
        Ms, params, nsite = args
        env = StateEnvs(psi0, H, Ms, weight=kwargs.pop("weight", -1.0))
    else:
        params, nsite = args
        env = StateEnvs(psi0, H)
    sw = dmrg_(env, params, nsite, **kwargs)
    return sw.energy[-1], env.getpsi()


def dmrg2(psi0: MPS, H: MPO, *args, **kwargs):
    """``dmrg2(psi0, H, [Ms,] params)`` (``src/mps/dmrg.jl:295-301``)."""
    return dmrg(psi0, H, *args, 2, **kwargs)


def dmrg1(psi0: MPS, H: MPO, *args, **kwargs):
    """``dmrg1(psi0, H, [Ms,] params)`` (``src/mps/dmrg.jl:314-320``): one-site DMRG (with
    noise > 0 each site's solution is split with its neighbour through the two-site
    density-matrix perturbation)."""
    return dmrg(psi0, H, *args, 1, **kwargs)


# ------------------------------------------------------------------------------------
# checkpoint / resume
# ------------------------------------------------------------------------------------

def _charge_mask(ql, pq, qr):
    return (np.asarray(ql)[:, None, None] + np.asarray(pq)[None, :, None]) == \
        np.asarray(qr)[None, None, :]


def checkpoint_arrays(tensors, links, phys_q, center, swdata: SweepData | None = None) -> dict:
    """Host arrays of a checkpoint: for every site only the entries its charges allow (the
    charge blocks, concatenated), the link and site charges, the orthogonality centre and the
    sweep history."""
    out = {"phys_q": np.asarray(phys_q, dtype=np.int32), "center": np.int64(center),
           "nsites": np.int64(len(tensors))}
    for i, t in enumerate(tensors):
        t = np.asarray(t, dtype=np.complex128 if np.iscomplexobj(t) else np.float64)
        out[f"shape_{i}"] = np.array(t.shape, dtype=np.int64)
        out[f"blocks_{i}"] = t[_charge_mask(links[i], phys_q, links[i + 1])]
    for i, q in enumerate(links):
        out[f"link_{i}"] = np.asarray(q, dtype=np.int32)
    if swdata is not None:
        out["sw_sweepcount"] = np.int64(swdata.sweepcount)
        for k in ("maxchi", "energy", "entropy", "maxtruncerr"):
            out[f"sw_{k}"] = np.asarray(getattr(swdata, k), dtype=np.float64)
        lens = [len(e) for e in swdata.lasteigs]
        out["sw_lasteigs_len"] = np.asarray(lens, dtype=np.int64)
        out["sw_lasteigs"] = (np.concatenate([np.asarray(e, dtype=np.float64) for e in swdata.lasteigs])
                              if lens else np.zeros(0))
        out["sw_stats"] = np.array(json.dumps(swdata.stats))
    return out


def arrays_from_checkpoint(z) -> tuple:
    """(tensors, links, phys_q, center, swdata or None) from checkpoint_arrays' dict."""
    n = int(z["nsites"])
    pq = np.asarray(z["phys_q"], dtype=np.int32)
    links = [np.asarray(z[f"link_{i}"], dtype=np.int32) for i in range(n + 1)]
    tensors = []
    for i in range(n):
        b = z[f"blocks_{i}"]
        t = np.zeros(tuple(int(x) for x in z[f"shape_{i}"]), dtype=b.dtype)
        t[_charge_mask(links[i], pq, links[i + 1])] = b
        tensors.append(t)
    sw = None
    if "sw_sweepcount" in z:
        sw = SweepData()
        sw.sweepcount = int(z["sw_sweepcount"])
        sw.maxchi = [int(x) for x in z["sw_maxchi"]]
        for k in ("energy", "entropy", "maxtruncerr"):
            setattr(sw, k, [float(x) for x in z[f"sw_{k}"]])
        lens, flat, o = z["sw_lasteigs_len"], z["sw_lasteigs"], 0
        sw.lasteigs = []
        for ln in lens:
            sw.lasteigs.append(np.asarray(flat[o:o + int(ln)]))
            o += int(ln)
        sw.stats = json.loads(str(z["sw_stats"]))
    return tensors, links, pq, int(z["center"]), sw


def save_checkpoint(path, psi, swdata: SweepData | None = None):
    """Write a checkpoint of a DMRG run to ``path`` (numpy .npz): the state (an ``MPS`` or
    the current state of a ``StateEnvs``) and the sweep history.  The reference restarts a
    simulation from a serialised ``StateEnvs`` (docs/src/mps/example_dmrg.md:76-78); here the
    environments are rebuilt from the state on resume."""
    if isinstance(psi, StateEnvs):
        psi = psi.getpsi()
    tensors = [psi.site(i) for i in range(psi.N)]
    links = [psi.link_charges(i) for i in range(psi.N + 1)]
    np.savez(path, **checkpoint_arrays(tensors, links, psi.phys_q, psi.center, swdata))


def load_checkpoint(path, ctx: Context | None = None):
    """(MPS, SweepData or None) from a checkpoint; continue with ``StateEnvs(psi, H)`` and the
    same ``SweepData``."""
    with np.load(path, allow_pickle=False) as z:
        tensors, links, pq, center, sw = arrays_from_checkpoint(z)
    return MPS(tensors, links, pq, center, ctx), sw


def svd_truncate(blocks, maxdim=INT32_MAX, mindim=1, cutoff=None, ctx: Context | None = None):
    """Block SVD + ITensors-style global truncation on explicit dense blocks.

    Returns (kept per block, singular values per block sorted descending, truncerr).
    """
    ctx = ctx or Context.default()
    cutoff = Float64_threshold() if cutoff is None else cutoff
    rows = np.array([b.shape[0] for b in blocks], dtype=np.int32)
    cols = np.array([b.shape[1] for b in blocks], dtype=np.int32)
    data = np.concatenate([np.asarray(b, dtype=np.float64).ravel(order="F") for b in blocks])
    ns = np.minimum(rows, cols)
    sv = np.zeros(int(ns.sum()))
    kept = np.zeros(len(blocks), dtype=np.int32)
    te = C.c_double()
    L.check(ctx.lib.tn_svd_truncate(ctx.h, len(blocks), rows.ctypes.data_as(L.i32p),
                                    cols.ctypes.data_as(L.i32p), data.ctypes.data_as(L.f64p),
                                    int(min(maxdim, INT32_MAX)), int(mindim), float(cutoff),
                                    kept.ctypes.data_as(L.i32p), sv.ctypes.data_as(L.f64p),
                                    C.byref(te)))
    out, o = [], 0
    for n in ns:
        out.append(sv[o:o + n].copy())
        o += n
    return kept, out, te.value
