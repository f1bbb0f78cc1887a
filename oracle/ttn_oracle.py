"""CPU oracle for the tree tensor network (TTN) sweep (TEST INFRASTRUCTURE ONLY).

This module is the oracle, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` may import it.  The
product path (``libtennet_cuda.so``) never calls into it.

Plain numpy FP64 restatement of TenNetLib's TTN ground-state path (no charge conservation):

* ``default_graph_sitenodes`` / ``_distribute_site_positions`` -- ``src/ttn/ttn_generators.jl:4-96``
* ``randomTTN`` (index dimensions, then ``isometrize_full!``) -- ``src/ttn/ttn_generators.jl:191-261``
* ``moveisometry_to_next!`` (QR, or SVD with truncation when cutoff > 0 or the link is
  larger than maxdim), ``isometrize!``, ``normalize!`` -- ``src/ttn/ttn.jl:216-382``
* ``LinkTensorsTTN(psi, M)`` and ``move_linktensors_to_next!`` -- ``src/ttn/linktensors.jl:63-118``,
  ``:233-261``; pieces whose term is complete on the moved-to side are summed into one local
  tensor, the others are kept per term (the reference's ``order(phidag) > 2`` test)
* ``product(env, psi, v)`` -- ``src/ttn/linktensors.jl:183-221``
* ``position!`` (isometrize, then move the environment along the same path) --
  ``src/ttn/state_envs_ttn.jl:120-141``
* ``update_position!`` with ``eig_solver`` -- ``src/ttn/update_site_ttn.jl:42-63``,
  ``src/base/solver.jl:23-43``
* ``fullsweep!`` (noise = 0 branch: path then reversed path, cutoff = -1; noise > 0
  branch: position with ``node_to_skip``, ``subspace_expand!`` toward the central node and
  ``expand_numiter`` updates with the widened maxdims) and ``default_sweeppath`` --
  ``src/ttn/sweep_ttn.jl:49-65``, ``:117-274``, ``src/ttn/update_site_ttn.jl:75-109``
* ``optimize!`` stage loop with the noise schedule -- ``src/ttn/optimize_ttn.jl:148-226``

Subspace-expansion padding: the reference draws it with ``random_itensor`` (Julia's RNG,
normal entries); here it is a counter-based stream shared bit for bit with the engine
(splitmix64, uniform entries in [-1, 1), ``padding_values``), then scaled to
noise * |tensor| as in the reference, so that GPU and oracle expand identically.

Conventions shared with the engine (``include/tennet.h``):

* nodes are the reference's (layer, index) labels; the engine numbers them in sorted order;
* a node tensor's legs are its physical sites in ascending order, then its neighbour nodes
  in ascending order;
* a Hamiltonian is a list of product terms ``(coef, [(site, op), ...])`` with distinct
  sites; ``op[s', s]`` is a d x d matrix.  This is a CouplingModel whose terms are not
  merged (``_initCouplingModel(...; merge = false)``, ``src/base/couplingmodel.jl:153-230``).
  The reference spreads |coef|^(1/k) over the k operators; here coef multiplies the
  operator on the lowest site: the same operator, rounded differently.
* ``graph.nodes`` is a Julia ``Set``: where the reference breaks ties by its iteration order
  (the eccentric central node), this restatement takes the smallest label.

Parity: the arithmetic of ITensors (contraction, ``qr``, ``svd``) and KrylovKit is not
part of the reference tree; QR and SVD gauges differ from LAPACK's, which changes no
energy.  The oracle is pinned against the free-fermion solution of the open transverse
field Ising chain (``tfim_exact_energy``) and exact diagonalisation.
"""
from __future__ import annotations

from collections import deque
from dataclasses import dataclass, field

import numpy as np

from oracle.tn_oracle import FLOAT64_THRESHOLD, eigsolve_lowest, svd_blocks_truncate

PAULI_X = np.array([[0.0, 1.0], [1.0, 0.0]])
PAULI_Z = np.array([[1.0, 0.0], [0.0, -1.0]])


# --------------------------------------------------------------------------------------
# tree generation (src/ttn/ttn_generators.jl, src/ttn/helper_internal_funcs.jl)
# --------------------------------------------------------------------------------------

def min_power2_ge(n: int) -> int:
    """``_minimum_power2_greater_than`` (helper_internal_funcs.jl:10-20)."""
    if n <= 0:
        raise ValueError("input must be a positive integer")
    p = 1
    while p < n:
        p <<= 1
    return p


def _tz(n: int) -> int:
    return (n & -n).bit_length() - 1


def distribute_site_positions(numsites: int, loc=None) -> list[int]:
    """``_distribute_site_positions`` (ttn_generators.jl:4-46): per layer-1 slot, 1 if a site
    sits there, 0 if not."""
    if not loc:
        rem = numsites % 2
        loc = [numsites // 2, numsites // 2 + rem]
        numsites = min_power2_ge(numsites)
    else:
        power = _tz(len(loc))
        newloc = []
        for m in loc:
            rem = m % 2
            newloc.append(m // 2 + rem if power % 2 == 1 else m // 2)
            newloc.append(m // 2 if power % 2 == 1 else m // 2 + rem)
        loc = newloc
    numsites //= 2
    if _tz(numsites) > 1:
        return distribute_site_positions(numsites, loc)
    pos = []
    for m in loc:
        if m == 1:
            pos += [1, 0]
        elif m == 2:
            pos += [1, 1]
        else:
            raise RuntimeError("_distribute_site_positions: inconsistent split")
    return pos


def default_graph_sitenodes(N: int):
    """``default_graph_sitenodes`` (ttn_generators.jl:69-96).

    Returns (adjacency dict node -> sorted neighbour list, site_nodes list: site (0-based) ->
    node).  Nodes are (layer, index) tuples with the reference's 1-based labels."""
    pos = distribute_site_positions(N)
    p2 = len(pos)
    nl = _tz(p2)
    adj: dict = {}

    def edge(a, b):
        adj.setdefault(a, set()).add(b)
        adj.setdefault(b, set()).add(a)

    site_nodes = []
    for ll in range(1, nl - 1):
        for nn in range(1, (p2 >> ll) + 1):
            if ll == 1 and (pos[2 * nn - 2] == 0 or pos[2 * nn - 1] == 0):
                site_nodes.append((ll + 1, (nn + 1) // 2))
                continue
            if ll == 1:
                site_nodes += [(ll, nn), (ll, nn)]
            edge((ll, nn), (ll + 1, (nn + 1) // 2))
    edge((nl - 1, 1), (nl - 1, 2))
    return {k: sorted(v) for k, v in sorted(adj.items())}, site_nodes


def default_sweeppath(N: int, nodes) -> list:
    """``default_sweeppath`` (sweep_ttn.jl:49-65)."""
    nsites = min_power2_ge(N)
    nl = _tz(nsites)
    path = []
    nodeset = set(nodes)
    for ll in range(nl - 1, 0, -1):
        cnt = nsites >> ll
        for nn in range(1, cnt + 1):
            nnpos = nn if (nl - ll) % 2 == 1 else cnt - nn + 1
            node = (ll, nnpos)
            if ll == 1 and node not in nodeset:
                continue
            path.append(node)
    return path


def bfs(adj, src):
    """``bfs`` (src/base/graph.jl:200-230): distances and parents."""
    dist, par = {src: 0}, {}
    q = deque([src])
    while q:
        x = q.popleft()
        for y in adj[x]:
            if y not in dist:
                dist[y] = dist[x] + 1
                par[y] = x
                q.append(y)
    return dist, par


def shortest_path(adj, a, b) -> list:
    """``shortest_path`` (src/base/graph.jl:293-312)."""
    if a == b:
        return [a]
    _, par = bfs(adj, a)
    out = [b]
    while out[-1] != a:
        out.append(par[out[-1]])
    return out[::-1]


def eccentric_center(adj, nodes=None):
    """``find_eccentric_central_node`` (src/base/graph.jl:413-431); ties -> smallest label."""
    best, bestd = None, None
    for v in sorted(adj):
        dist, _ = bfs(adj, v)
        dd = max(dist[x] for x in (nodes if nodes is not None else dist))
        if bestd is None or dd < bestd:
            best, bestd = v, dd
    return best


def nodes_from_bfs_reverse(adj, src) -> list:
    """``nodes_from_bfs(graph, src; reverse = true)``: farthest first (ties: label order)."""
    dist, _ = bfs(adj, src)
    return sorted(dist, key=lambda v: (-dist[v], v))


# --------------------------------------------------------------------------------------
# the TTN state
# --------------------------------------------------------------------------------------

@dataclass
class TTN:
    adj: dict                 # node -> sorted neighbour list
    site_nodes: list          # site -> node
    d: int
    tensors: dict = field(default_factory=dict)
    center: tuple | None = None

    @property
    def nodes(self):
        return sorted(self.adj)

    def sites_of(self, v):
        return [n for n, x in enumerate(self.site_nodes) if x == v]

    def legs(self, v):
        """Leg labels of node v: ('s', site) for its sites, then ('n', neighbour)."""
        return [("s", n) for n in self.sites_of(v)] + [("n", u) for u in self.adj[v]]

    def leg_index(self, v, u):
        return self.legs(v).index(("n", u))

    def link_dim(self, v, u):
        return self.tensors[v].shape[self.leg_index(v, u)]

    def maxlinkdim(self):
        """``maxlinkdim`` (ttn.jl:199-209)."""
        md = 1
        for v in self.adj:
            for u in self.adj[v]:
                md = max(md, self.link_dim(v, u))
        return md

    def copy(self):
        return TTN(self.adj, self.site_nodes, self.d,
                   {k: t.copy() for k, t in self.tensors.items()}, self.center)

    def subtree_sites(self, v, u):
        """Sites on v's side of the edge (v, u)."""
        seen, stack, out = {u, v}, [v], []
        while stack:
            x = stack.pop()
            out += self.sites_of(x)
            for y in self.adj[x]:
                if y not in seen:
                    seen.add(y)
                    stack.append(y)
        return set(out)


def _matricize(T, leg):
    """(rest, leg) matrix of T with the rest legs in order; returns it and a restorer."""
    Tm = np.moveaxis(T, leg, -1)
    shp = Tm.shape
    return Tm.reshape(-1, shp[-1]), shp


def move_isometry(psi: TTN, v, u, maxdim=2**62, mindim=1, cutoff=1e-15):
    """``moveisometry_to_next!`` (ttn.jl:266-310): QR unless cutoff > 0 or the link is
    larger than maxdim, then an SVD with ITensors truncation."""
    A = psi.tensors[v]
    lv = psi.leg_index(v, u)
    Am, shp = _matricize(A, lv)
    if cutoff > 0.0 or Am.shape[1] > maxdim:
        out, _spec, _kept = svd_blocks_truncate([Am], maxdim, mindim, cutoff)
        Uk, Sk, Vk = out[0]
        Q, R = Uk, Sk[:, None] * Vk
    else:
        Q, R = np.linalg.qr(Am, mode="reduced")
    k = Q.shape[1]
    psi.tensors[v] = np.moveaxis(Q.reshape(shp[:-1] + (k,)), -1, lv)
    B = psi.tensors[u]
    lu = psi.leg_index(u, v)
    psi.tensors[u] = np.moveaxis(np.tensordot(R, B, axes=([1], [lu])), 0, lu)
    psi.center = u


def normalize_ttn(psi: TTN):
    """``normalize!`` (ttn.jl:216-222)."""
    c = psi.center
    psi.tensors[c] = psi.tensors[c] / np.linalg.norm(psi.tensors[c])


def isometrize_full(psi: TTN, node, normalize=True, **kw):
    """``isometrize_full!`` (ttn.jl:326-346)."""
    for v in nodes_from_bfs_reverse(psi.adj, node)[:-1]:
        move_isometry(psi, v, shortest_path(psi.adj, v, node)[1], **kw)
    psi.center = node
    if normalize:
        normalize_ttn(psi)


def isometrize(psi: TTN, node, normalize=True, **kw):
    """``isometrize!`` (ttn.jl:359-382)."""
    path = shortest_path(psi.adj, psi.center, node)
    for a, b in zip(path[:-1], path[1:]):
        move_isometry(psi, a, b, **kw)
    if normalize:
        normalize_ttn(psi)


def random_ttn(N: int, chi: int, seed: int, d: int = 2) -> TTN:
    """``default_randomTTN`` / ``randomTTN`` (ttn_generators.jl:191-281) without charges:
    link dimensions min(product of the node's other legs, chi) built from the leaves
    toward the eccentric centre, Gaussian entries from numpy's PCG64 stream ``seed`` (node
    by node in label order), then ``isometrize_full!`` with cutoff 0 and maxdim chi."""
    adj, site_nodes = default_graph_sitenodes(N)
    psi = TTN(adj, site_nodes, d)
    center = eccentric_center(adj, set(site_nodes))
    dims = {}
    for v in adj:
        dims[v] = {("s", n): d for n in psi.sites_of(v)}
    for v in nodes_from_bfs_reverse(adj, center)[:-1]:
        nxt = shortest_path(adj, v, center)[1]
        D = min(int(np.prod(list(dims[v].values()))), chi)
        dims[v][("n", nxt)] = D
        dims[nxt][("n", v)] = D
    rng = np.random.default_rng(seed)
    for v in psi.nodes:
        shape = tuple(dims[v][leg] for leg in psi.legs(v))
        t = rng.standard_normal(shape)
        psi.tensors[v] = t / np.linalg.norm(t)
    isometrize_full(psi, center, normalize=True, cutoff=0.0, maxdim=chi)
    return psi


# --------------------------------------------------------------------------------------
# Hamiltonians (product terms)
# --------------------------------------------------------------------------------------

def tfim_terms(J, h):
    """Open transverse-field Ising chain H = -sum_i J_i Z_i Z_{i+1} - sum_i h_i X_i."""
    N = len(h)
    terms = [(-float(J[i]), [(i, PAULI_Z), (i + 1, PAULI_Z)]) for i in range(N - 1)]
    terms += [(-float(h[i]), [(i, PAULI_X)]) for i in range(N)]
    return terms


def tfim_instance(N: int, seed: int):
    """One random instance: J_i ~ U[0.5, 1.5], uniform h ~ U[0.8, 1.2]."""
    rng = np.random.default_rng(seed)
    J = rng.uniform(0.5, 1.5, size=N - 1)
    h = np.full(N, rng.uniform(0.8, 1.2))
    return J, h


def heisenberg_terms(N: int):
    """S=1/2 Heisenberg chain sum_i S_i . S_{i+1} as product terms."""
    sz = np.diag([0.5, -0.5])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    out = []
    for i in range(N - 1):
        out.append((1.0, [(i, sz), (i + 1, sz)]))
        out.append((0.5, [(i, sp), (i + 1, sm)]))
        out.append((0.5, [(i, sm), (i + 1, sp)]))
    return out


def tfim_exact_energy(J, h) -> float:
    """Ground energy of the open TFIM by Jordan-Wigner: minus the sum of the singular values
    of the bidiagonal matrix with diagonal h_i and superdiagonal J_i (Lieb, Schultz, Mattis
    1961; Pfeuty 1970)."""
    N = len(h)
    B = np.diag(np.asarray(h, dtype=np.float64))
    for i in range(N - 1):
        B[i, i + 1] = J[i]
    return -float(np.sum(np.linalg.svd(B, compute_uv=False)))


def dense_hamiltonian(N: int, terms, d: int = 2) -> np.ndarray:
    """Dense H (site 0 = most significant factor); for exact checks at small N."""
    H = np.zeros((d**N, d**N))
    for coef, ops in terms:
        mats = [np.eye(d)] * N
        for s, o in ops:
            mats[s] = o
        M = mats[0]
        for m in mats[1:]:
            M = np.kron(M, m)
        H += coef * M
    return H


def ttn_to_dense(psi: TTN) -> np.ndarray:
    """Contract the TTN into the full state vector (site 0 most significant)."""
    nodes = psi.nodes
    # label every leg; contract with einsum
    letters = iter("abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ")
    lab, ops, subs = {}, [], []
    for v in nodes:
        s = ""
        for leg in psi.legs(v):
            key = ("s", leg[1]) if leg[0] == "s" else ("e",) + tuple(sorted([v, leg[1]]))
            if key not in lab:
                lab[key] = next(letters)
            s += lab[key]
        ops.append(psi.tensors[v])
        subs.append(s)
    out = "".join(lab[("s", n)] for n in range(len(psi.site_nodes)))
    return np.einsum(",".join(subs) + "->" + out, *ops, optimize=True).reshape(-1)


# --------------------------------------------------------------------------------------
# link tensors (src/ttn/linktensors.jl)
# --------------------------------------------------------------------------------------

def _apply_leg(x, M, leg):
    """(M x_leg x)[.., a', ..] = sum_a M[a', a] x[.., a, ..]."""
    return np.moveaxis(np.tensordot(M, x, axes=([1], [leg])), 0, leg)


class LinkEnv:
    """``LinkTensorsTTN`` without charges.  ``links[key]`` holds the tensors of one link
    oriented toward the side of the current orthogonality centre: ``{"local": M or None,
    "open": {term: M}}``; key ("s", n) for the site links, frozenset({v, u}) for tree links.
    """

    def __init__(self, psi: TTN, terms):
        self.terms = terms
        self.term_sites = [frozenset(s for s, _ in ops) for _, ops in terms]
        self.links = {}
        N = len(psi.site_nodes)
        for n in range(N):
            local, opn = None, {}
            for t, (coef, ops) in enumerate(terms):
                for j, (s, o) in enumerate(ops):
                    if s != n:
                        continue
                    first = min(x for x, _ in ops) == n
                    m = (coef * o) if first else o.copy()
                    if len(ops) == 1:
                        local = m if local is None else local + m
                    else:
                        opn[t] = m
            self.links[("s", n)] = {"local": local, "open": opn}
        # LinkTensorsTTN(psi, M) (linktensors.jl:233-261): from the leaves toward the centre
        oc = psi.center
        for v in nodes_from_bfs_reverse(psi.adj, oc)[:-1]:
            self.move_to_next(psi, v, shortest_path(psi.adj, v, oc)[1])

    def _groups(self, psi: TTN, v, skip=None):
        """Per term (or per local piece) the (leg, matrix) list of node v's links."""
        groups = []
        byterm = {}
        for li, leg in enumerate(psi.legs(v)):
            if leg[0] == "n" and leg[1] == skip:
                continue
            key = ("s", leg[1]) if leg[0] == "s" else frozenset({v, leg[1]})
            if key not in self.links:
                continue
            ent = self.links[key]
            if ent["local"] is not None:
                groups.append((None, [(li, ent["local"])]))
            for t, M in ent["open"].items():
                byterm.setdefault(t, []).append((li, M))
        for t in sorted(byterm):
            groups.append((t, byterm[t]))
        return groups

    def move_to_next(self, psi: TTN, v, u):
        """``move_linktensors_to_next!`` (linktensors.jl:63-118)."""
        phi = psi.tensors[v]
        lu = psi.leg_index(v, u)
        side = psi.subtree_sites(v, u)
        local, opn = None, {}
        for t, pieces in self._groups(psi, v, skip=u):
            y = phi
            for li, M in pieces:
                y = _apply_leg(y, M, li)
            rest = [i for i in range(phi.ndim) if i != lu]
            T = np.tensordot(phi, y, axes=(rest, rest))  # [a', a]
            if t is None or self.term_sites[t] <= side:
                local = T if local is None else local + T
            else:
                opn[t] = T
        self.links[frozenset({v, u})] = {"local": local, "open": opn}

    def product(self, psi: TTN, v, x):
        """``product(env, psi, v)`` (linktensors.jl:183-221) at node v."""
        out = np.zeros_like(x)
        for _t, pieces in self._groups(psi, v):
            y = x
            for li, M in pieces:
                y = _apply_leg(y, M, li)
            out += y
        return out


class LinkProj:
    """``LinkProjTTN`` (src/ttn/linkproj.jl:15-224) without charges: ``E[(v, u)]`` is the
    overlap of psi and M on v's side of the link (v, u), indexed [a_psi, a_M]
    (``move_linkproj_to_next!``, linkproj.jl:56-78); the projected vector at the centre
    contracts M's centre tensor with the overlaps of all its links (``contract``,
    linkproj.jl:143-157)."""

    def __init__(self, psi: TTN, M: TTN):
        self.M = M.copy()
        self.E = {}
        oc = psi.center
        for v in nodes_from_bfs_reverse(psi.adj, oc)[:-1]:
            self.move_to_next(psi, v, shortest_path(psi.adj, v, oc)[1])

    def _mapped(self, psi: TTN, v, skip):
        y = self.M.tensors[v].conj()
        for li, leg in enumerate(psi.legs(v)):
            if leg[0] == "n" and leg[1] != skip and (leg[1], v) in self.E:
                y = _apply_leg(y, self.E[(leg[1], v)], li)
        return y

    def move_to_next(self, psi: TTN, v, u):
        y = self._mapped(psi, v, u)
        lu = psi.leg_index(v, u)
        rest = [i for i in range(y.ndim) if i != lu]
        self.E[(v, u)] = np.tensordot(psi.tensors[v], y, axes=(rest, rest))  # [a_psi, a_M]

    def vector(self, psi: TTN, v):
        return self._mapped(psi, v, None)


# --------------------------------------------------------------------------------------
# StateEnvsTTN, update, sweeps
# --------------------------------------------------------------------------------------

@dataclass
class SweepDataTTN:
    """``SweepDataTTN`` (sweep_ttn.jl:4-26)."""
    sweepcount: int = 0
    maxchi: list = field(default_factory=list)
    energy: list = field(default_factory=list)


# --------------------------------------------------------------------------------------
# subspace expansion (noise > 0)
# --------------------------------------------------------------------------------------

def _splitmix64(x):
    """splitmix64 of a uint64 array (wrapping arithmetic)."""
    x = x + np.uint64(0x9E3779B97F4A7C15)
    z = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def padding_values(seed, event, instance, which, n):
    """n values in [-1, 1): value j is the top 53 bits of splitmix64(key + j) scaled, with
    key = splitmix64(seed + 2 (4096 event + instance) + which) (which: 0 for the node's
    padding, 1 for the next node's) -- the engine's stream, bit for bit."""
    with np.errstate(over="ignore"):
        base = np.array([seed], dtype=np.uint64) + np.array(
            [2 * (4096 * event + instance) + which], dtype=np.uint64)
        key = _splitmix64(base)
        x = _splitmix64(key + np.arange(n, dtype=np.uint64))
    return (x >> np.uint64(11)).astype(np.float64) * 2.0 ** -52 - 1.0


def subspace_expand(psi: TTN, node, nextnode, max_expand_dim, noise, seed, event, instance=0):
    """``subspace_expand!`` (src/ttn/update_site_ttn.jl:75-109): the link (node, nextnode)
    grows by pad = min(sum of the other leg dims of each tensor, max_expand_dim)
    (``indexintersection``, src/base/helper_internal_funcs.jl:182-188); each tensor gets a
    random block along it scaled to noise * its norm (direct sum, old components first)."""
    A, B = psi.tensors[node], psi.tensors[nextnode]
    la, lb = psi.leg_index(node, nextnode), psi.leg_index(nextnode, node)
    pad = min(sum(A.shape) - A.shape[la], sum(B.shape) - B.shape[lb], max_expand_dim)
    if pad <= 0:
        return 0
    for which, (v, T, leg) in enumerate(((node, A, la), (nextnode, B, lb))):
        shp = list(T.shape)
        shp[leg] = pad
        P = padding_values(seed, event, instance, which, int(np.prod(shp))).reshape(shp,
                                                                                    order="F")
        P *= noise * np.linalg.norm(T) / np.linalg.norm(P)
        psi.tensors[v] = np.concatenate([T, P], axis=leg)
    return pad


class StateEnvsTTN:
    """``StateEnvsTTN(psi, M)`` (state_envs_ttn.jl:27-31); with ``Ms`` and ``weight`` the
    projected environment ``EnvCouplingModelProjTTN`` (src/ttn/environment.jl:44-110):
    H_eff x + weight sum_k m_k (m_k . x)."""

    def __init__(self, psi: TTN, terms, Ms=None, weight=None):
        self.psi = psi.copy()
        self.env = LinkEnv(self.psi, terms)
        self.proj = []
        self.weight = 0.0
        if Ms:
            if weight is None or weight <= 0.0:
                raise ValueError("`weight` parameter should be > 0.0 (value passed was "
                                 f"`weight={weight}`)")
            self.proj = [LinkProj(self.psi, M) for M in Ms]
            self.weight = float(weight)
        self.expand_events = 0  # subspace expansions so far (the padding stream's counter)

    def position(self, node, normalize=True, maxdim=2**62, mindim=1, cutoff=1e-15,
                 node_to_skip=None):
        """``position!`` (state_envs_ttn.jl:120-141); the link moves out of
        ``node_to_skip`` are left out (``move_linktensors!``, linktensors.jl:130-154)."""
        oc = self.psi.center
        isometrize(self.psi, node, normalize=normalize, maxdim=maxdim, mindim=mindim,
                   cutoff=cutoff)
        path = shortest_path(self.psi.adj, oc, node)
        for a, b in zip(path[:-1], path[1:]):
            if a == node_to_skip:
                continue
            self.env.move_to_next(self.psi, a, b)
            for P in self.proj:
                P.move_to_next(self.psi, a, b)

    def product(self, x):
        out = self.env.product(self.psi, self.psi.center, x)
        for P in self.proj:
            m = P.vector(self.psi, self.psi.center)
            out = out + self.weight * m * float(np.vdot(m, x))
        return out


def update_position(se: StateEnvsTTN, node, maxdim=2**62, mindim=1, cutoff=-1.0,
                    normalize=True, krylovdim=5, maxiter=2, tol=1e-14):
    """``update_position!`` (update_site_ttn.jl:42-63) with ``eig_solver``."""
    se.position(node, normalize=normalize, maxdim=maxdim, mindim=mindim, cutoff=cutoff)
    phi = se.psi.tensors[node]
    shape = phi.shape
    e, vec, info = eigsolve_lowest(lambda y: se.product(y.reshape(shape)).reshape(-1),
                                   phi.reshape(-1), krylovdim, maxiter, tol)
    se.psi.tensors[node] = vec.reshape(shape)
    return e, info


def fullsweep(se: StateEnvsTTN, path, sw: SweepDataTTN, maxdim=2**62, mindim=1,
              krylovdim=5, maxiter=2, tol=1e-14, noise=0.0, cutoff=FLOAT64_THRESHOLD,
              expand_dim=None, max_expand_dim=None, expand_numiter=4, seed=0, instance=0):
    """``fullsweep!`` (sweep_ttn.jl:117-274).  noise below 100 Float64_threshold: every node
    of path and of the reversed path is updated with cutoff = -1 (QR moves).  Otherwise each
    node but the eccentric central one is expanded toward the central node: position there
    (QR moves, the link move out of the next node left out), ``subspace_expand!`` of the
    link, the centre set to the next node, then expand_numiter updates alternating node and
    next node with maxdims maxdim + max_expand_dim, maxdim + expand_dim, ..., maxdim and the
    given cutoff (SVD moves)."""
    sw.sweepcount += 1
    e = float("nan")
    kw = dict(krylovdim=krylovdim, maxiter=maxiter, tol=tol)
    if abs(noise) < 100 * FLOAT64_THRESHOLD:
        for node in list(path) + list(reversed(path)):
            e, _ = update_position(se, node, maxdim=maxdim, mindim=mindim, cutoff=-1.0, **kw)
    else:
        if expand_dim is None:
            expand_dim = 20
        if max_expand_dim is None:
            max_expand_dim = 2 * expand_dim
        if expand_dim != 0 and expand_numiter < 2:
            raise ValueError(f"`fullsweep!()`: `expand_numiter={expand_numiter}` cannot be "
                             f"less than 2 for `expand_dim={expand_dim}` !!")
        adj = se.psi.adj
        central = eccentric_center(adj)
        for node in list(path) + list(reversed(path)):
            if node == central:
                e, _ = update_position(se, node, maxdim=maxdim, mindim=mindim, cutoff=-1.0,
                                       **kw)
                continue
            nxt = shortest_path(adj, node, central)[1]
            se.position(node, normalize=True, maxdim=maxdim, mindim=mindim, cutoff=-1.0,
                        node_to_skip=nxt)
            subspace_expand(se.psi, node, nxt, max_expand_dim, noise, seed, se.expand_events,
                            instance)
            se.expand_events += 1
            se.psi.center = nxt
            for it in range(1, expand_numiter + 1):
                md = (maxdim if it == expand_numiter else
                      maxdim + max_expand_dim if it == 1 else maxdim + expand_dim)
                e, _ = update_position(se, node if it % 2 == 1 else nxt, maxdim=md,
                                       mindim=mindim, cutoff=cutoff, **kw)
    sw.maxchi.append(se.psi.maxlinkdim())
    sw.energy.append(e)
    return (sw.energy[-1] - sw.energy[-2]) if sw.sweepcount > 1 else float("nan")


def optimize(se: StateEnvsTTN, maxdims, nsweeps, path, energy_err_goal=None, cutoff=None,
             noise=0.0, noisedecay=1.0, disable_noise_after=2**62, **kw):
    """``optimize!`` (optimize_ttn.jl:148-226): stages of (maxdim, nsweeps) with the noise
    schedule (noise divided by noisedecay after each sweep, zero after disable_noise_after
    sweeps of a stage or below 100 Float64_threshold)."""
    sw = SweepDataTTN()
    n = len(nsweeps)

    def vec(x):
        return list(x) if isinstance(x, (list, tuple)) else [x] * n

    cutoffs = vec(FLOAT64_THRESHOLD if cutoff is None else cutoff)
    noises, decays, offs = vec(noise), vec(noisedecay), vec(disable_noise_after)
    for ii, (md, ns) in enumerate(zip(maxdims, nsweeps)):
        nz = noises[ii]
        for jj in range(1, ns + 1):
            de = fullsweep(se, path, sw, maxdim=md, noise=nz, cutoff=cutoffs[ii], **kw)
            if (energy_err_goal is not None and abs(de) < abs(energy_err_goal)
                    and abs(nz) < FLOAT64_THRESHOLD):
                break
            if jj == offs[ii]:
                nz = 0.0
            nz /= decays[ii]
            if nz < 100 * FLOAT64_THRESHOLD:
                nz = 0.0
    return sw
