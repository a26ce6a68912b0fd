"""CSR graph description shared by the GPU library and its callers.

A network of ``nv`` vertices is stored as an adjacency list in CSR form:

* vertex ``u`` owns legs ``off[u] .. off[u+1]-1``; leg slot ``s`` is the *directed*
  edge ``u -> nbr[s]`` with bond dimension ``bond[s]``;
* ``rev[s]`` is the slot of the opposite direction ``nbr[s] -> u``;
* site tensor of ``u`` is row-major ``[phys][leg_0]...[leg_{z-1}]`` (legs in CSR order)
  and lives at ``toff[u] .. toff[u+1]`` of one packed array;
* the message on slot ``s`` lives at ``moff[s] .. moff[s+1]`` of one packed array:
  for a norm network (``layers=2``) it is the ``D x D`` operator ``m[bra][ket]``
  (message_environment, messagecache.jl:205-229: codomain = bra link, domain = ket
  link), for a plain network (``layers=1``) a length-``D`` vector.

This mirrors how the reference identifies legs with edges: the link indices of an
edge are the dim names two vertex tensors share (abstracttensornetwork.jl:52-73),
and several shared names between one pair of vertices fuse into one leg.

Generators here produce the seeded synthetic inputs used by tests and benchmarks
(square lattices, random 3-regular graphs, combs/paths for tree tests).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Graph:
    nv: int
    off: np.ndarray
    nbr: np.ndarray
    bond: np.ndarray
    rev: np.ndarray
    phys: np.ndarray
    layers: int = 2
    net: np.ndarray | None = None  # network id per vertex (batched networks)
    toff: np.ndarray = field(init=False)
    moff: np.ndarray = field(init=False)

    def __post_init__(self):
        self.off = np.asarray(self.off, dtype=np.int64)
        self.nbr = np.asarray(self.nbr, dtype=np.int64)
        self.bond = np.asarray(self.bond, dtype=np.int32)
        self.rev = np.asarray(self.rev, dtype=np.int64)
        self.phys = np.asarray(self.phys, dtype=np.int32)
        if self.net is None:
            self.net = np.zeros(self.nv, dtype=np.int32)
        self.net = np.asarray(self.net, dtype=np.int32)
        sizes = np.empty(self.nv, dtype=np.int64)
        for u in range(self.nv):
            sizes[u] = int(self.phys[u]) * int(np.prod(self.bond[self.off[u]:self.off[u + 1]],
                                                      dtype=np.int64))
        self.toff = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        msz = self.bond.astype(np.int64) ** (2 if self.layers == 2 else 1)
        self.moff = np.concatenate([[0], np.cumsum(msz)]).astype(np.int64)

    # --- basic facts ---------------------------------------------------------------
    @property
    def nslots(self) -> int:
        return int(self.off[-1])

    @property
    def n_nets(self) -> int:
        """Number of networks (at least one, as the C ABI counts an empty network as one)."""
        return int(self.net.max()) + 1 if self.nv else 1

    def degree(self, u: int) -> int:
        return int(self.off[u + 1] - self.off[u])

    def legs(self, u: int) -> list[int]:
        return [int(b) for b in self.bond[self.off[u]:self.off[u + 1]]]

    def slot(self, u: int, w: int) -> int:
        """Slot of the directed edge u -> w (first one if there are several)."""
        for s in range(self.off[u], self.off[u + 1]):
            if self.nbr[s] == w:
                return int(s)
        raise KeyError((u, w))

    def slot_src(self, s: int) -> int:
        return int(np.searchsorted(self.off, s, side="right") - 1)

    def undirected_slots(self) -> np.ndarray:
        s = np.arange(self.nslots)
        return s[s < self.rev]

    def tensor_shape(self, u: int) -> tuple:
        return (int(self.phys[u]),) + tuple(self.legs(u))

    def message_shape(self, s: int) -> tuple:
        D = int(self.bond[s])
        return (D, D) if self.layers == 2 else (D,)

    def with_layers(self, layers: int) -> "Graph":
        return Graph(self.nv, self.off, self.nbr, self.bond, self.rev, self.phys, layers,
                     self.net)

    def with_phys(self, phys) -> "Graph":
        p = np.full(self.nv, phys, dtype=np.int32) if np.isscalar(phys) else phys
        return Graph(self.nv, self.off, self.nbr, self.bond, self.rev, p, self.layers,
                     self.net)


def from_edges(nv: int, edges, bonds, phys=2, layers=2, net=None) -> Graph:
    """Build a CSR graph from an undirected edge list ``[(u, w), ...]``.

    Legs of each vertex appear in the order its edges occur in ``edges``.
    ``bonds`` is one int (uniform) or one int per edge."""
    edges = [(int(a), int(b)) for a, b in edges]
    if np.isscalar(bonds):
        bonds = [int(bonds)] * len(edges)
    adj = [[] for _ in range(nv)]  # (nbr, bond, edge id, end)
    for e, ((a, b), D) in enumerate(zip(edges, bonds)):
        if a == b:
            raise ValueError("self loops are not supported")
        adj[a].append((b, int(D), e, 0))
        adj[b].append((a, int(D), e, 1))
    off = np.zeros(nv + 1, dtype=np.int64)
    for u in range(nv):
        off[u + 1] = off[u] + len(adj[u])
    ns = int(off[-1])
    nbr = np.zeros(ns, dtype=np.int64)
    bond = np.zeros(ns, dtype=np.int32)
    rev = np.zeros(ns, dtype=np.int64)
    where = {}
    for u in range(nv):
        for j, (w, D, e, end) in enumerate(adj[u]):
            s = off[u] + j
            nbr[s] = w
            bond[s] = D
            where[(e, end)] = s
    for (e, end), s in where.items():
        rev[s] = where[(e, 1 - end)]
    ph = np.full(nv, phys, dtype=np.int32) if np.isscalar(phys) else np.asarray(phys)
    return Graph(nv, off, nbr, bond, rev, ph, layers, net)


def square_lattice_edges(Lx: int, Ly: int, periodic: bool = False):
    """Edges of an Lx x Ly square lattice, vertex id = x * Ly + y.  Each vertex's legs
    come out in the order (x-1 side, y-1 side, y+1 side, x+1 side) for the bulk."""
    if periodic and (Lx < 3 or Ly < 3):
        raise ValueError("periodic lattices need Lx, Ly >= 3 (no double edges)")
    edges = []
    for x in range(Lx):
        for y in range(Ly):
            u = x * Ly + y
            if y + 1 < Ly or periodic:
                edges.append((u, x * Ly + (y + 1) % Ly))
            if x + 1 < Lx or periodic:
                edges.append((u, ((x + 1) % Lx) * Ly + y))
    return edges


def square_lattice(Lx, Ly, D, *, periodic=False, phys=2, layers=2) -> Graph:
    return from_edges(Lx * Ly, square_lattice_edges(Lx, Ly, periodic), D, phys, layers)


def random_regular_edges(n: int, k: int, rng: np.random.Generator, max_tries: int = 1000):
    """Simple k-regular graph on n vertices by the pairing model with rejection."""
    if (n * k) % 2:
        raise ValueError("n * k must be even")
    for _ in range(max_tries):
        stubs = np.repeat(np.arange(n), k)
        rng.shuffle(stubs)
        pairs = stubs.reshape(-1, 2)
        if np.any(pairs[:, 0] == pairs[:, 1]):
            continue
        key = np.sort(pairs, axis=1)
        if len(np.unique(key[:, 0] * n + key[:, 1])) != len(key):
            continue
        return [(int(a), int(b)) for a, b in key]
    raise RuntimeError("could not draw a simple regular graph")


def path_edges(n: int):
    return [(i, i + 1) for i in range(n - 1)]


def cycle_edges(n: int):
    return [(i, (i + 1) % n) for i in range(n)]


def comb_tree_edges(nx: int, ny: int):
    """Comb: a backbone (x, 0) for x < nx, each with a tooth (x, 1..ny-1).
    Vertex id = x * ny + y (like a grid of the same shape)."""
    edges = []
    for x in range(nx):
        if x + 1 < nx:
            edges.append((x * ny, (x + 1) * ny))
        for y in range(ny - 1):
            edges.append((x * ny + y, x * ny + y + 1))
    return edges


def batched(graphs: list[Graph]) -> Graph:
    """Disjoint union of several networks; ``net`` records the network of each vertex."""
    layers = graphs[0].layers
    offs, nbrs, bonds, revs, phys, nets = [np.zeros(1, dtype=np.int64)], [], [], [], [], []
    vbase = 0
    sbase = 0
    for i, g in enumerate(graphs):
        if g.layers != layers:
            raise ValueError("all networks need the same layer count")
        offs.append(g.off[1:] + sbase)
        nbrs.append(g.nbr + vbase)
        bonds.append(g.bond)
        revs.append(g.rev + sbase)
        phys.append(g.phys)
        nets.append(np.full(g.nv, i, dtype=np.int32))
        vbase += g.nv
        sbase += g.nslots
    return Graph(vbase, np.concatenate(offs), np.concatenate(nbrs), np.concatenate(bonds),
                 np.concatenate(revs), np.concatenate(phys), layers, np.concatenate(nets))


# --- seeded synthetic inputs ------------------------------------------------------------

def random_tensors(g: Graph, rng: np.random.Generator, dtype=np.float64, scale=None):
    """Packed site tensors with iid N(0,1) entries (complex: N(0,1) + i N(0,1)), each
    tensor scaled by ``scale`` (callable u -> factor, a float, or None)."""
    n = int(g.toff[-1])
    dt = np.dtype(dtype)
    if dt.kind == "c":
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    else:
        x = rng.standard_normal(n)
    if scale is not None:
        if callable(scale):
            for u in range(g.nv):
                x[g.toff[u]:g.toff[u + 1]] *= scale(u)
        else:
            x *= scale
    return x.astype(dt)


def peps_scale(g: Graph):
    """1/sqrt(d * prod(bond dims)) per vertex: 1/sqrt(d*D^4) on a square lattice."""
    def f(u):
        return 1.0 / np.sqrt(float(g.toff[u + 1] - g.toff[u]))
    return f


def identity_messages(g: Graph, dtype=np.float64, normalized=True):
    """message_environment(one, nn) (messagecache.jl:227-229), optionally divided by the
    sum of entries (identity / D) as the first update's normalisation would do."""
    m = np.zeros(int(g.moff[-1]), dtype=dtype)
    for s in range(g.nslots):
        D = int(g.bond[s])
        blk = np.eye(D, dtype=dtype) if g.layers == 2 else np.ones(D, dtype=dtype)
        if normalized:
            blk = blk / blk.sum()
        m[g.moff[s]:g.moff[s + 1]] = blk.ravel()
    return m


def ones_messages(g: Graph, dtype=np.float64):
    return np.ones(int(g.moff[-1]), dtype=dtype)


def random_messages(g: Graph, rng, dtype=np.float64):
    """rand(rng, T, dims) entries in [0, 1) (test_beliefpropagation.jl:211-213)."""
    dt = np.dtype(dtype)
    n = int(g.moff[-1])
    if dt.kind == "c":
        return (rng.random(n) + 1j * rng.random(n)).astype(dt)
    return rng.random(n).astype(dt)


def tree_edge_sequence(g: Graph, root: int = 0) -> np.ndarray:
    """Directed-slot schedule that makes one sequential sweep exact on a forest:
    leaves-to-root (post-order) then root-to-leaves, per connected component.
    Plays the role of forest_cover_edge_sequence on trees (beliefpropagation.jl:14);
    on graphs with cycles it is applied to a BFS spanning forest and the remaining
    edges are appended in both directions."""
    seen = np.zeros(g.nv, dtype=bool)
    up = []  # slots child -> parent, in post-order
    used = np.zeros(g.nslots, dtype=bool)
    roots = [root] + [u for u in range(g.nv) if u != root]
    for r in roots:
        if seen[r]:
            continue
        seen[r] = True
        order = []
        stack = [(r, -1)]
        parent_slot = {}
        while stack:
            u, ps = stack.pop()
            order.append(u)
            for s in range(g.off[u], g.off[u + 1]):
                w = int(g.nbr[s])
                if not seen[w]:
                    seen[w] = True
                    parent_slot[w] = int(g.rev[s])  # slot w -> u
                    stack.append((w, s))
        for u in reversed(order):
            if u in parent_slot:
                up.append(parent_slot[u])
    for s in up:
        used[s] = True
        used[g.rev[s]] = True
    down = [int(g.rev[s]) for s in reversed(up)]
    rest = [s for s in range(g.nslots) if not used[s]]
    return np.asarray(up + down + rest, dtype=np.int64)
