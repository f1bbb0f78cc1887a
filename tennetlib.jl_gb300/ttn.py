"""Tree tensor networks (TTN): TenNetLib's TTN ground-state path on one GB300.

=================================  ===========================================================
Python                              TenNetLib (file:line)
=================================  ===========================================================
``default_graph_sitenodes(N)``      ``default_graph_sitenodes``   src/ttn/ttn_generators.jl:69-96
``default_randomTTN(N, chi, seed)`` ``default_randomTTN``         src/ttn/ttn_generators.jl:273-281
``TTN``                             ``TTN``                       src/ttn/ttn.jl:21-26
``TTN.isometrize_``                 ``isometrize!``               src/ttn/ttn.jl:359-382
``CouplingModel(terms, N)``         ``CouplingModel``             src/base/couplingmodel.jl:246-300
``StateEnvsTTN(psi, H)``            ``StateEnvsTTN``              src/ttn/state_envs_ttn.jl:27-31
``StateEnvsTTN.position_``          ``position!``                 src/ttn/state_envs_ttn.jl:120-141
``StateEnvsTTN.product``            ``product``                   src/ttn/linktensors.jl:183-221
``update_position_``                ``update_position!``          src/ttn/update_site_ttn.jl:42-63
``fullsweep_``                      ``fullsweep!``                src/ttn/sweep_ttn.jl:117-274
``SweepDataTTN``                    ``SweepDataTTN``              src/ttn/sweep_ttn.jl:4-26
``default_sweeppath(psi)``          ``default_sweeppath``         src/ttn/sweep_ttn.jl:49-65
``OptimizeParamsTTN``               ``OptimizeParamsTTN``         src/ttn/optimize_ttn.jl:25-110
``optimize_`` / ``optimize``        ``optimize!`` / ``optimize``  src/ttn/optimize_ttn.jl:148-281
``measure(psi, op[, pos])``         ``measure``                   src/ttn/measure_ttn.jl:12-170
=================================  ===========================================================

Beyond the reference: ``StateEnvsTTN.batch(psis, models)`` creates environments that share
one device arena, and ``fullsweep_batch_`` sweeps them in lockstep (one grouped launch per
contraction stage for all of them) -- the reference runs independent instances one after
the other.

Sites are 0-based; nodes keep the reference's (layer, index) labels.  The tree logic here
is integer bookkeeping; the floating-point work runs in libtennet_cuda.so (``measure``'s
last contraction of one node tensor with a d x d operator is done on the host).
"""
from __future__ import annotations

import ctypes as C
import math
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


def _own(obj, handle):
    from . import _own as own
    own(obj, handle)


def _release(obj, name):
    from . import _release as rel
    rel(obj, name)

INT32_MAX = 2**31 - 1
PAULI_X = np.array([[0.0, 1.0], [1.0, 0.0]])
PAULI_Z = np.array([[1.0, 0.0], [0.0, -1.0]])


# --------------------------------------------------------------------------------------
# the default hierarchical binary tree
# --------------------------------------------------------------------------------------

def _pow2_ge(n: int) -> int:
    if n <= 0:
        raise ValueError("number of sites must be positive")
    return 1 << (n - 1).bit_length()


def _tz(n: int) -> int:
    return (n & -n).bit_length() - 1


def _site_slots(n: int, loc=None):
    """Per layer-1 slot of the padded binary tree: 1 where a site sits, 0 where none
    (``_distribute_site_positions``, src/ttn/ttn_generators.jl:4-46)."""
    if not loc:
        loc = [n // 2, n // 2 + n % 2]
        n = _pow2_ge(n)
    else:
        odd = _tz(len(loc)) % 2 == 1
        nxt = []
        for m in loc:
            lo, hi = m // 2, m // 2 + m % 2
            nxt += [hi, lo] if odd else [lo, hi]
        loc = nxt
    n //= 2
    if _tz(n) > 1:
        return _site_slots(n, loc)
    out = []
    for m in loc:
        if m not in (1, 2):
            raise RuntimeError("site distribution failed")
        out += [1, 0] if m == 1 else [1, 1]
    return out


def default_graph_sitenodes(N: int):
    """(graph, sitenodes): adjacency {label: sorted neighbour labels} of the default binary
    tree for N sites and the node label of each site (0-based list)."""
    if N < 5:
        raise ValueError("the default tree needs at least 5 sites (with 4 or fewer the "
                         "reference's generator attaches no site)")
    slots = _site_slots(N)
    p2 = len(slots)
    nl = _tz(p2)
    adj: dict = {}
    sitenodes = []
    for ll in range(1, nl - 1):
        for nn in range(1, (p2 >> ll) + 1):
            if ll == 1 and (slots[2 * nn - 2] == 0 or slots[2 * nn - 1] == 0):
                sitenodes.append((2, (nn + 1) // 2))
                continue
            if ll == 1:
                sitenodes += [(1, nn), (1, nn)]
            a, b = (ll, nn), (ll + 1, (nn + 1) // 2)
            adj.setdefault(a, set()).add(b)
            adj.setdefault(b, set()).add(a)
    a, b = (nl - 1, 1), (nl - 1, 2)
    adj.setdefault(a, set()).add(b)
    adj.setdefault(b, set()).add(a)
    return {k: sorted(v) for k, v in sorted(adj.items())}, sitenodes


def _bfs(adj, src):
    dist = {src: 0}
    q = deque([src])
    while q:
        x = q.popleft()
        for y in adj[x]:
            if y not in dist:
                dist[y] = dist[x] + 1
                q.append(y)
    return dist


def eccentric_central_node(adj, nodes=None):
    """``find_eccentric_central_node`` (src/base/graph.jl:413-431); ties -> smallest label."""
    best, bestd = None, None
    for v in sorted(adj):
        dist = _bfs(adj, v)
        dd = max(dist[x] for x in (nodes if nodes is not None else dist))
        if bestd is None or dd < bestd:
            best, bestd = v, dd
    return best


def default_sweeppath(psi) -> list:
    """``default_sweeppath`` (src/ttn/sweep_ttn.jl:49-65)."""
    N = psi.N if hasattr(psi, "N") else int(psi)
    nodes = set(psi.labels) if hasattr(psi, "labels") else set(default_graph_sitenodes(N)[0])
    nsites = _pow2_ge(N)
    nl = _tz(nsites)
    path = []
    for ll in range(nl - 1, 0, -1):
        cnt = nsites >> ll
        for nn in range(1, cnt + 1):
            node = (ll, nn if (nl - ll) % 2 == 1 else cnt - nn + 1)
            if ll == 1 and node not in nodes:
                continue
            path.append(node)
    return path


# --------------------------------------------------------------------------------------
# TTN state
# --------------------------------------------------------------------------------------

class TTN:
    """A TTN on the device (``TTN{T}``, src/ttn/ttn.jl:21-26), dense node tensors.

    ``graph``: {label: neighbour labels}; ``sitenodes``: node label of each site; node
    tensor legs: the node's sites ascending, then its neighbours in label order."""

    def __init__(self, graph, sitenodes, d, tensors=None, center=None, ctx=None, _handle=None):
        from . import Context  # noqa: F811
        self.ctx = ctx or Context.default()
        self.graph = {k: list(v) for k, v in graph.items()}
        self.labels = sorted(self.graph)
        self.index = {v: i for i, v in enumerate(self.labels)}
        self.sitenodes = list(sitenodes)
        self.N = len(self.sitenodes)
        self.d = d
        self.edges = sorted({tuple(sorted((self.index[a], self.index[b])))
                             for a in self.graph for b in self.graph[a]})
        if _handle is not None:
            _own(self, _handle)
            return
        dims = {}
        for e in self.edges:
            a, b = self.labels[e[0]], self.labels[e[1]]
            ta = np.asarray(tensors[a])
            dims[e] = ta.shape[self.legs(a).index(("n", b))]
        flat = np.concatenate([np.asarray(tensors[v], dtype=np.float64).ravel(order="F")
                               for v in self.labels])
        ed = np.array(self.edges, dtype=np.int32).ravel()
        sn = np.array([self.index[x] for x in self.sitenodes], dtype=np.int32)
        ld = np.array([dims[e] for e in self.edges], dtype=np.int32)
        c = -1 if center is None else self.index[center]
        bufs = [L.as_i32(ed), L.as_i32(sn), L.as_i32(ld), L.as_f64(flat)]
        h = L.vp()
        L.check(self.ctx.lib.tn_ttn_create(self.ctx.h, self.N, d, len(self.labels), len(self.edges),
                                           bufs[0][1], bufs[1][1], bufs[2][1], bufs[3][1], c,
                                           C.byref(h)))
        _own(self, h)

    def sites_of(self, v):
        return [n for n, x in enumerate(self.sitenodes) if x == v]

    def legs(self, v):
        return [("s", n) for n in self.sites_of(v)] + [("n", u) for u in self.graph[v]]

    @property
    def orthocenter(self):
        c = self.ctx.lib.tn_ttn_center(self.h)
        return None if c < 0 else self.labels[c]

    def node_dims(self, v):
        n = C.c_int32()
        dims = np.zeros(64, dtype=np.int32)
        L.check(self.ctx.lib.tn_ttn_node_dims(self.h, self.index[v], C.byref(n),
                                              dims.ctypes.data_as(L.i32p)))
        return tuple(int(x) for x in dims[: n.value])

    def __getitem__(self, v):
        shape = self.node_dims(v)
        out = np.zeros(int(np.prod(shape)))
        L.check(self.ctx.lib.tn_ttn_node(self.h, self.index[v], out.ctypes.data_as(L.f64p),
                                         out.size))
        return out.reshape(shape, order="F")

    def tensors(self):
        return {v: self[v] for v in self.labels}

    def maxlinkdim(self):
        return int(self.ctx.lib.tn_ttn_maxlinkdim(self.h))

    def isometrize_(self, node, normalize=True):
        """``isometrize!`` with QR moves (``isometrize_full!`` when there is no centre)."""
        L.check(self.ctx.lib.tn_ttn_isometrize(self.h, self.index[node], int(bool(normalize))))
        return self

    def __del__(self):
        try:
            _release(self, "tn_ttn_destroy")
        except Exception:
            pass


def random_ttn_tensors(N: int, chi: int, seed: int, d: int = 2):
    """(graph, sitenodes, tensors, centre) of ``randomTTN``'s construction
    (src/ttn/ttn_generators.jl:191-261) without charges: link dimension min(product of the
    node's other legs, chi) from the leaves toward the eccentric centre; Gaussian entries
    from numpy's PCG64 stream ``seed``, node by node in label order, each tensor
    normalised.  Not yet an isometric TTN."""
    graph, sitenodes = default_graph_sitenodes(N)
    center = eccentric_central_node(graph, set(sitenodes))
    dist = _bfs(graph, center)
    par = {}
    for v in graph:
        for u in graph[v]:
            if dist[u] == dist[v] - 1:
                par[v] = u
    dims = {v: {("s", n): d for n, x in enumerate(sitenodes) if x == v} for v in graph}
    for v in sorted(graph, key=lambda x: (-dist[x], x)):
        if v == center:
            continue
        D = min(int(np.prod(list(dims[v].values()))), chi)
        dims[v][("n", par[v])] = D
        dims[par[v]][("n", v)] = D
    rng = np.random.default_rng(seed)
    tensors = {}
    for v in sorted(graph):
        legs = [("s", n) for n, x in enumerate(sitenodes) if x == v] + [("n", u) for u in graph[v]]
        t = rng.standard_normal(tuple(dims[v][g] for g in legs))
        tensors[v] = t / np.linalg.norm(t)
    return graph, sitenodes, tensors, center


def default_randomTTN(N: int, chi: int, seed: int, d: int = 2, ctx=None) -> TTN:
    """``default_randomTTN(sites, chi)``: random tensors, then ``isometrize_full!`` toward
    the eccentric centre on the GPU (QR moves) and normalisation."""
    graph, sitenodes, tensors, center = random_ttn_tensors(N, chi, seed, d)
    psi = TTN(graph, sitenodes, d, tensors, None, ctx)
    return psi.isometrize_(center, normalize=True)


# --------------------------------------------------------------------------------------
# Hamiltonian
# --------------------------------------------------------------------------------------

class CouplingModel:
    """Sum of product terms ``[(coef, [(site, op), ...]), ...]`` (``CouplingModel`` with
    unmerged terms, src/base/couplingmodel.jl:153-230); op is a d x d matrix [s', s]."""

    def __init__(self, terms, N: int, d: int = 2):
        self.terms = terms
        self.N = N
        self.d = d
        nops, sites, ops, coef = [], [], [], []
        for c, fs in terms:
            nops.append(len(fs))
            coef.append(float(c))
            for s, o in fs:
                sites.append(int(s))
                ops.append(np.asarray(o, dtype=np.float64).ravel(order="F"))
        self._bufs = [L.as_i32(nops), L.as_i32(sites),
                      L.as_f64(np.concatenate(ops) if ops else np.zeros(1)), L.as_f64(coef)]
        self.lib = L.load()
        h = L.vp()
        L.check(self.lib.tn_ttn_model_create(N, d, len(terms), self._bufs[0][1], self._bufs[1][1],
                                             self._bufs[2][1], self._bufs[3][1], C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.lib.tn_ttn_model_destroy(self.h)
        except Exception:
            pass


def _op_matrix(op, d):
    from . import SPIN_HALF_OPS
    if isinstance(op, str):
        if d != 2 or op not in SPIN_HALF_OPS:
            raise ValueError(f"unknown operator name {op!r} (S=1/2 names: {sorted(SPIN_HALF_OPS)})")
        return SPIN_HALF_OPS[op]
    m = np.asarray(op, dtype=np.float64)
    if m.shape != (d, d):
        raise ValueError("an operator must be a d x d matrix [s', s]")
    return m


def measure(psi: TTN, op, pos=None, sites=None):
    """``measure(T, psi, opstr[, pos]; sites)`` (src/ttn/measure_ttn.jl:12-86): <O_i> at every
    site (or ``pos``, or ``sites``; 0-based) -- for each node holding such sites the centre is
    moved there (``isometrize!`` with QR moves on the GPU, normalised; psi is changed as in the
    reference) and O contracted with its tensor.  With a list of (operator, site) pairs,
    ``measure(T, psi, ["Sz" => i, "Sz" => j, ...])`` (:96-170): the centre is moved to the
    eccentric central node of the sites' nodes and <psi| O_i O_j ... |psi> is the product of
    the link tensors of that one product term (``LinkTensorsTTN(psi, optens)``, GPU) with the
    centre tensor.  Operators are S=1/2 names or d x d matrices; fermionic Jordan-Wigner
    strings (``isfermions``) are not applied."""
    if isinstance(op, (list, tuple)) and op and isinstance(op[0], (list, tuple)):
        return _measure_product(psi, op)
    mat = _op_matrix(op, psi.d)
    targets = [int(pos)] if pos is not None else (
        [int(x) for x in sites] if sites is not None else list(range(psi.N)))
    bynode = {}
    for site in targets:
        bynode.setdefault(psi.sitenodes[site], []).append(site)
    out = {}
    for node, ss in bynode.items():
        psi.isometrize_(node)
        T = psi[node]
        legs = psi.legs(node)
        for site in ss:
            li = legs.index(("s", site))
            y = np.moveaxis(np.tensordot(mat, T, axes=([1], [li])), 0, li)
            out[site] = float(np.vdot(T, y))
    vals = [out[site] for site in targets]
    return vals[0] if pos is not None else vals


def _measure_product(psi: TTN, oppairs):
    ops = {}
    for name, site in oppairs:
        m = _op_matrix(name, psi.d)
        site = int(site)
        ops[site] = ops[site] @ m if site in ops else m  # O_a(i) O_b(i) -> the product A B
    model = CouplingModel([(1.0, [(site, ops[site]) for site in sorted(ops)])], psi.N, psi.d)
    oc = eccentric_central_node(psi.graph, {psi.sitenodes[site] for site in ops})
    psi.isometrize_(oc)
    env = StateEnvsTTN(psi, model)
    x = psi[oc]
    return float(np.vdot(x, env.product(x)))


def tfim_terms(J, h):
    """Open transverse-field Ising chain H = -sum_i J_i Z_i Z_{i+1} - sum_i h_i X_i."""
    N = len(h)
    out = [(-float(J[i]), [(i, PAULI_Z), (i + 1, PAULI_Z)]) for i in range(N - 1)]
    out += [(-float(h[i]), [(i, PAULI_X)]) for i in range(N)]
    return out


def tfim_instance(N: int, seed: int):
    """Random couplings J_i ~ U[0.5, 1.5] and one uniform field h ~ U[0.8, 1.2]."""
    rng = np.random.default_rng(seed)
    J = rng.uniform(0.5, 1.5, size=N - 1)
    h = np.full(N, rng.uniform(0.8, 1.2))
    return J, h


def heisenberg_terms(N: int):
    """S=1/2 Heisenberg chain sum_i S_i . S_{i+1} as product terms."""
    sz = np.diag([0.5, -0.5])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    out = []
    for i in range(N - 1):
        out += [(1.0, [(i, sz), (i + 1, sz)]), (0.5, [(i, sp), (i + 1, sp.T)]),
                (0.5, [(i, sp.T), (i + 1, sp)])]
    return out


# --------------------------------------------------------------------------------------
# environments and sweeps
# --------------------------------------------------------------------------------------

class StateEnvsTTN:
    """``StateEnvsTTN(psi, H)``: a copy of psi and its link tensors on the device.

    ``StateEnvsTTN(psi, H, Ms, weight=w)`` (src/ttn/state_envs_ttn.jl:36-52) adds the
    excited-state projectors of the states ``Ms``: products and updates then use
    H_eff + w sum_k |m_k><m_k| (EnvCouplingModelProjTTN, src/ttn/environment.jl:104-110)."""

    def __init__(self, psi: TTN, H: CouplingModel, Ms=None, *, weight=None, _handle=None):
        self.ctx = psi.ctx
        self.template = psi
        self.H = H
        if _handle is not None:
            _own(self, _handle)
            return
        hs = (L.vp * 1)()
        L.check(self.ctx.lib.tn_ttn_envs_create(1, (L.vp * 1)(psi.h), (L.vp * 1)(H.h), hs))
        _own(self, L.vp(hs[0]))
        if Ms is not None:
            self.set_projectors(Ms, -1.0 if weight is None else weight)

    def set_projectors(self, Ms, weight: float):
        """Projectors onto the states ``Ms`` (copied) with weight > 0; ``[]`` removes them."""
        Ms = list(Ms)
        self._Ms = Ms
        arr = (L.vp * max(len(Ms), 1))(*[m.h for m in Ms])
        L.check(self.ctx.lib.tn_ttn_env_set_projectors(self.h, arr, len(Ms), float(weight)))
        return self

    @classmethod
    def batch(cls, psis, models):
        """Environments of several states sharing one device arena, for
        ``fullsweep_batch_``; all states share one tree and centre."""
        n = len(psis)
        hs = (L.vp * n)()
        L.check(psis[0].ctx.lib.tn_ttn_envs_create(n, (L.vp * n)(*[p.h for p in psis]),
                                                   (L.vp * n)(*[m.h for m in models]), hs))
        return [cls(p, m, _handle=L.vp(hs[i])) for i, (p, m) in enumerate(zip(psis, models))]

    def getpsi(self) -> TTN:
        h = L.vp()
        L.check(self.ctx.lib.tn_ttn_env_getpsi(self.h, C.byref(h)))
        t = self.template
        return TTN(t.graph, t.sitenodes, t.d, ctx=self.ctx, _handle=h)

    @property
    def psi(self) -> TTN:
        return self.getpsi()

    @property
    def orthocenter(self):
        return self.template.labels[self.ctx.lib.tn_ttn_env_center(self.h)]

    def position_(self, node):
        L.check(self.ctx.lib.tn_ttn_env_position(self.h, self.template.index[node]))
        return self

    def product(self, v):
        v = np.asarray(v, dtype=np.float64)
        flat = np.ascontiguousarray(v.ravel(order="F"))
        out = np.zeros_like(flat)
        L.check(self.ctx.lib.tn_ttn_env_product(self.h, flat.ctypes.data_as(L.f64p),
                                                out.ctypes.data_as(L.f64p), flat.size))
        return out.reshape(v.shape, order="F")

    __call__ = product

    def product_flops(self) -> float:
        f = C.c_double()
        L.check(self.ctx.lib.tn_ttn_env_product_flops(self.h, C.byref(f)))
        return f.value

    def __del__(self):
        try:
            _release(self, "tn_ttn_env_destroy")
        except Exception:
            pass


def _params(kwargs) -> L.UpdateParams:
    p = L.UpdateParams()
    p.maxdim = int(min(kwargs.get("maxdim", INT32_MAX), INT32_MAX))
    p.mindim = int(kwargs.get("mindim", 1))
    p.cutoff = -1.0
    p.normalize = int(bool(kwargs.get("normalize", True)))
    p.krylovdim = int(kwargs.get("solver_krylovdim", 5))
    p.maxiter = int(kwargs.get("solver_maxiter", 2))
    p.tol = float(kwargs.get("solver_tol", 1e-14))
    p.eager = int(bool(kwargs.get("solver_eager", False)))
    p.check_convergence = int(bool(kwargs.get("solver_check_convergence", False)))
    p.noise = float(kwargs.get("noise", 0.0))
    if kwargs.get("time_step") is not None:
        raise ValueError("time_step is reserved for future use in the reference (sweep_ttn.jl:126)")
    return p


def _eig_solver_token(solver):
    from . import eig_solver
    if solver is not eig_solver:
        raise ValueError("only eig_solver is supported (src/ttn/sweep_ttn.jl:83)")


def update_position_(sysenv: StateEnvsTTN, solver, node, **kwargs):
    """``update_position!`` (src/ttn/update_site_ttn.jl:42-63); returns the energy."""
    _eig_solver_token(solver)
    p = _params(kwargs)
    r = L.UpdateResult()
    L.check(sysenv.ctx.lib.tn_ttn_env_update_position(sysenv.h, sysenv.template.index[node],
                                                      C.byref(p), C.byref(r)))
    return r.energy


@dataclass
class SweepDataTTN:
    """``SweepDataTTN`` (src/ttn/sweep_ttn.jl:4-26) plus device timings per sweep."""
    sweepcount: int = 0
    maxchi: list = field(default_factory=list)
    energy: list = field(default_factory=list)
    stats: list = field(default_factory=list)


def _stats(r: L.SweepResult):
    return {k: getattr(r, k) for k, _ in L.SweepResult._fields_}


def fullsweep_batch_(envs, sweeppath, solver, swdatas, **kwargs):
    """``fullsweep!`` (src/ttn/sweep_ttn.jl:117-274) on environments made by
    ``StateEnvsTTN.batch`` (or one environment), in lockstep; returns the energy changes.
    noise >= 100 Float64_threshold takes the subspace-expansion branch (``expand_dim``
    default 20, ``max_expand_dim`` 2 expand_dim, ``expand_numiter`` 4, ``cutoff`` the SVD
    cutoff of its updates, ``seed`` of the padding stream)."""
    from . import Float64_threshold
    _eig_solver_token(solver)
    t = envs[0].template
    path = np.array([t.index[v] for v in sweeppath], dtype=np.int32)
    p = _params(kwargs)
    n = len(envs)
    res = (L.SweepResult * n)()
    hs = (L.vp * n)(*[e.h for e in envs])
    noise = float(kwargs.get("noise", 0.0))
    if abs(noise) < 100 * Float64_threshold():
        p.noise = 0.0
        L.check(envs[0].ctx.lib.tn_ttn_envs_fullsweep(n, hs, len(path),
                                                      path.ctypes.data_as(L.i32p), C.byref(p),
                                                      res))
    else:
        expand_dim = int(kwargs.get("expand_dim", 20))
        max_expand_dim = int(kwargs.get("max_expand_dim", 2 * expand_dim))
        numiter = int(kwargs.get("expand_numiter", 4))
        p.cutoff = float(kwargs.get("cutoff", Float64_threshold()))
        central = t.index[eccentric_central_node(t.graph)]
        L.check(envs[0].ctx.lib.tn_ttn_envs_fullsweep_expand(
            n, hs, len(path), path.ctypes.data_as(L.i32p), central, C.byref(p), expand_dim,
            max_expand_dim, numiter, int(kwargs.get("seed", 0)) & (2 ** 64 - 1), res))
    out = []
    for sw, r in zip(swdatas, res):
        sw.sweepcount += 1
        sw.maxchi.append(int(r.maxlinkdim))
        sw.energy.append(float(r.energy))
        sw.stats.append(_stats(r))
        out.append(sw.energy[-1] - sw.energy[-2] if sw.sweepcount > 1 else math.nan)
        if kwargs.get("outputlevel", 1) > 0:
            print(f"At sweep {sw.sweepcount} => E={sw.energy[-1]}, MaxLinkDim={sw.maxchi[-1]}")
    return out


def fullsweep_(sysenv: StateEnvsTTN, sweeppath, solver, swdata: SweepDataTTN, **kwargs):
    """``fullsweep!`` (src/ttn/sweep_ttn.jl:117-274)."""
    return fullsweep_batch_([sysenv], sweeppath, solver, [swdata], **kwargs)[0]


@dataclass
class OptimizeParamsTTN:
    """``OptimizeParamsTTN`` (src/ttn/optimize_ttn.jl:25-110)."""
    maxdim: list
    nsweeps: list
    cutoff: object = 1e-15
    noise: object = 0.0
    noisedecay: object = 1.0
    disable_noise_after: object = INT32_MAX

    def __post_init__(self):
        n = len(self.nsweeps)
        vec = lambda x: list(x) if isinstance(x, (list, tuple)) else [x] * n
        self.cutoff, self.noise = vec(self.cutoff), vec(self.noise)
        self.noisedecay, self.disable_noise_after = vec(self.noisedecay), vec(self.disable_noise_after)
        if not (len(self.maxdim) == n == len(self.cutoff) == len(self.noise) ==
                len(self.noisedecay) == len(self.disable_noise_after)):
            raise ValueError("OptimizeParamsTTN: size mismatch in input vectors")


def optimize_(sysenv, params: OptimizeParamsTTN, sweeppath, **kwargs) -> SweepDataTTN:
    """``optimize!`` (src/ttn/optimize_ttn.jl:148-226): the stages of params with the noise
    schedule (noise divided by noisedecay after every sweep, zero after disable_noise_after
    sweeps of a stage or below 100 Float64_threshold)."""
    from . import Float64_threshold, eig_solver
    goal = kwargs.pop("energyErrGoal", None)
    sw = SweepDataTTN()
    for ii in range(len(params.nsweeps)):
        noise = float(params.noise[ii])
        for jj in range(1, params.nsweeps[ii] + 1):
            de = fullsweep_(sysenv, sweeppath, eig_solver, sw, maxdim=params.maxdim[ii],
                            cutoff=params.cutoff[ii], noise=noise, **kwargs)
            if goal is not None and abs(de) < abs(goal) and abs(noise) < Float64_threshold():
                break
            if jj == params.disable_noise_after[ii]:
                noise = 0.0
            noise /= params.noisedecay[ii]
            if noise < 100 * Float64_threshold():
                noise = 0.0
    return sw


def optimize(psi0: TTN, H: CouplingModel, *args, **kwargs):
    """``optimize(psi0, H, params, sweeppath)`` or, for an excited state,
    ``optimize(psi0, H, Ms, params, sweeppath; weight)`` (src/ttn/optimize_ttn.jl:274-301):
    returns (energy, psi)."""
    if len(args) == 3:
        Ms, params, sweeppath = args
        weight = kwargs.pop("weight", -1.0)
        se = StateEnvsTTN(psi0, H, Ms, weight=weight)
    elif len(args) == 2:
        params, sweeppath = args
        se = StateEnvsTTN(psi0, H)
    else:
        raise TypeError("optimize(psi0, H, [Ms,] params, sweeppath)")
    sw = optimize_(se, params, sweeppath, **kwargs)
    return sw.energy[-1], se.getpsi()
