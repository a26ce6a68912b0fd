"""The reference's named-tensor API, mirrored over the GPU engine.

ITensorNetworksNext.jl works with named tensors (ITensorBase ``ITensor``s whose axes carry
index names), networks whose edges are the names two tensors share, and message caches
keyed by directed edges.  This module gives the same objects and entry points in Python:

=========================================  ==================================================
reference (ITensorNetworksNext.jl)         here
=========================================  ==================================================
``Index``, ``ITensor``                     ``Index``, ``ITensor`` (numpy data + indices)
``ITensorNetwork``, ``tensornetwork``      ``ITensorNetwork`` (src/tensornetwork.jl:21-48)
``NormNetwork``, ``normnetwork``           ``NormNetwork`` (src/normnetwork.jl:13-93)
``MessageCache``, ``messagecache``         ``MessageCache`` (messagecache.jl:15-52)
``message_environment(f, nn)``             ``message_environment`` (messagecache.jl:205-229)
``beliefpropagation(factors, messages;     ``beliefpropagation`` (beliefpropagation.jl:69-92)
edges, stopping_criterion, alg)``
``message_update!(cache, factors, edge)``  ``message_update`` (beliefpropagation.jl:230-257)
``iterate_diff``                           ``iterate_diff`` (beliefpropagation.jl:261-267)
``vertex_scalar(s)``, ``edge_scalar(s)``,  same names (messagecache.jl:139-201)
``region_scalar``, ``bethe_free_energy``
``contract_network(tn; alg=Exact())``      ``contract_network`` (contract_network.jl:7-58)
=========================================  ==================================================

Every computation runs on the GPU through libitn_gpu.so: the network is flattened to the
CSR layout of the C ABI (all names shared by two vertices fuse into one leg, all site names
of a vertex into its physical axis) and results are unflattened back onto named tensors.
There is no CPU fallback.  ``SimpleMessageUpdate`` keeps the reference's sequential
(Gauss-Seidel) sweep over ``edges``; ``GPUMessageUpdate`` adds the parallel (Jacobi)
schedule and the tensor-core precision modes.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

from . import graphs as G
from ._lib import ItnArgumentError
from .contract import contract_network as _contract_arrays
from .engine import BPEngine

_uid = itertools.count()


# ---- named tensors ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Index:
    """An index: a dimension with a name (fresh unique name by default)."""
    dim: int
    name: object = field(default_factory=lambda: ("i", next(_uid)))

    def __repr__(self):
        return f"Index({self.dim}, {self.name!r})"


def uniquename(name=None):
    return ("u", next(_uid))


class ITensor:
    """Dense array with one Index per axis."""

    def __init__(self, data, inds):
        data = np.asarray(data)
        inds = tuple(inds)
        if data.ndim != len(inds) or any(d != i.dim for d, i in zip(data.shape, inds)):
            raise ValueError("data shape does not match the indices")
        self.data = data
        self.inds = inds

    @property
    def dimnames(self):
        return tuple(i.name for i in self.inds)

    def permute(self, names):
        """Data with axes in the order of ``names``."""
        pos = [self.dimnames.index(n) for n in names]
        return np.transpose(self.data, pos)

    def conj(self):
        return ITensor(np.conj(self.data), self.inds)

    def replacenames(self, f):
        return ITensor(self.data, [Index(i.dim, f(i.name)) for i in self.inds])

    def __getitem__(self, _):
        """``t[]`` of a scalar tensor."""
        return self.data[()]

    def __repr__(self):
        return f"ITensor({self.data.shape}, {self.dimnames})"


def itensor(data, *inds):
    return ITensor(data, inds)


# ---- networks ---------------------------------------------------------------------------------
class ITensorNetwork:
    """Vertex -> ITensor; an edge joins two vertices that share an index name
    (set!_tensornetwork, src/tensornetwork.jl:138-173)."""

    def __init__(self, tensors):
        self.tensors = dict(tensors)
        self._vs = list(self.tensors)
        owners = {}
        for v in self._vs:
            for n in self.tensors[v].dimnames:
                owners.setdefault(n, []).append(v)
        for n, vs in owners.items():
            if len(vs) > 2:
                raise ValueError(f"index name {n!r} is shared by more than two tensors")
        self.dimname_vertices = owners

    def vertices(self):
        return list(self._vs)

    def __getitem__(self, v):
        return self.tensors[v]

    def __setitem__(self, v, t):
        self.tensors[v] = t
        self.__init__(self.tensors)

    def linknames(self, u, v):
        """Names shared by u and v (linknames, abstracttensornetwork.jl:69-73)."""
        nv = set(self.tensors[v].dimnames)
        return [n for n in self.tensors[u].dimnames if n in nv]

    def sitenames(self, v):
        return [n for n in self.tensors[v].dimnames if len(self.dimname_vertices[n]) == 1]

    def neighbors(self, v):
        out = []
        for n in self.tensors[v].dimnames:
            for w in self.dimname_vertices[n]:
                if w != v and w not in out:
                    out.append(w)
        return out

    def edges(self):
        seen, out = set(), []
        for v in self._vs:
            for w in self.neighbors(v):
                if (w, v) not in seen:
                    seen.add((v, w))
                    out.append((v, w))
        return out


def tensornetwork(f, vertices):
    return ITensorNetwork({v: f(v) for v in vertices})


class NormNetwork:
    """<tn|tn> with a ket -> bra name map for link names; site names map to themselves
    (NormNetwork, src/normnetwork.jl:13-25, braname :66-73)."""

    def __init__(self, ket: ITensorNetwork, braname=None):
        self.ket = ket
        self.braname = {}
        for n, vs in ket.dimname_vertices.items():
            if len(vs) == 2:
                self.braname[n] = braname[n] if braname is not None else uniquename(n)

    def vertices(self):
        return self.ket.vertices()

    def edges(self):
        return self.ket.edges()

    def bra(self, name):
        return self.braname.get(name, name)

    def kettensor(self, v):
        return self.ket[v]

    def conj_bratensor(self, v):
        return self.ket[v].replacenames(self.bra)

    def bratensor(self, v):
        return self.conj_bratensor(v).conj()


def normnetwork(tn: ITensorNetwork, braname=None):
    return NormNetwork(tn, braname)


class _NormView:
    """A read-only view of one layer of a NormNetwork with its graph structure
    (KetView / BraView, src/normnetworkview.jl:6-58)."""

    def __init__(self, parent: NormNetwork):
        self.parent = parent

    def vertices(self):
        return self.parent.vertices()

    def edges(self):
        return self.parent.edges()

    def is_vertex_assigned(self, v):
        return v in self.parent.ket.tensors

    def issettable(self):
        return False

    def isinsertable(self):
        return False

    def __setitem__(self, v, t):
        raise TypeError(f"{type(self).__name__} is a read-only view of a NormNetwork")


class KetView(_NormView):
    """The ket layer: view[v] is kettensor(nn, v) itself."""

    def __getitem__(self, v):
        return self.parent.kettensor(v)

    def linknames(self, u, v):
        return self.parent.ket.linknames(u, v)


class BraView(_NormView):
    """The bra layer: view[v] is bratensor(nn, v) (link names mapped by braname, data
    conjugated)."""

    def __getitem__(self, v):
        return self.parent.bratensor(v)

    def linknames(self, u, v):
        return [self.parent.bra(n) for n in self.parent.ket.linknames(u, v)]


# ---- message caches -----------------------------------------------------------------------------
class MessageCache:
    """Directed edge (u, v) -> message ITensor (src/beliefpropagation/messagecache.jl:15-52)."""

    def __init__(self, messages):
        self.messages = dict(messages)

    def __getitem__(self, e):
        return self.messages[tuple(e)]

    def __setitem__(self, e, m):
        self.messages[tuple(e)] = m

    def edges(self):
        return list(self.messages)

    def keys(self):
        return self.messages.keys()

    def copy(self):
        return MessageCache(self.messages)

    def copyto(self, src, edges=None):
        """copyto!(dst, src[, edges]) of the DataGraphs interface that MessageCache implements
        (messagecache.jl:84-101; exercised by test/test_beliefpropagation.jl:63-81): src is
        another cache, a dict or a list of (edge, message) pairs; with ``edges``, only those
        directed edges of the cache ``src`` are copied.  In place; returns self."""
        if edges is not None:
            for e in edges:
                self.messages[tuple(e)] = src[tuple(e)]
            return self
        items = src.messages.items() if isinstance(src, MessageCache) else (
            src.items() if isinstance(src, dict) else src)
        for e, m in items:
            self.messages[tuple(e)] = m
        return self

    def __len__(self):
        return len(self.messages)


def messagecache(f_or_pairs, edges=None):
    if edges is None:
        return MessageCache(dict(f_or_pairs))
    return MessageCache({tuple(e): f_or_pairs(e) for e in edges})


def incoming_messages(cache: MessageCache, edge):
    """Messages into src(edge) except the reverse one (messagecache.jl:124-131)."""
    u, v = edge
    return [cache[e] for e in cache.edges() if e[1] == u and e[0] != v]


def insertlink(tn: ITensorNetwork, e):
    """insertlink!(tn, e) (abstracttensornetwork.jl:121-133): joins the two vertices of the
    edge e by a new link of dimension 1 (an all-ones factor on both tensors); in place,
    returns tn."""
    u, v = e
    link = Index(1, uniquename())
    for w in (u, v):
        t = tn.tensors[w]
        tn.tensors[w] = ITensor(t.data[..., None], list(t.inds) + [link])
    tn.__init__(tn.tensors)
    return tn


def message_environment(f, nn: NormNetwork):
    """One D x D operator per directed edge (codomain = bra link, domain = ket link),
    mapped by f: ``"one"`` -> identity, ``"ones"`` -> all ones, or a callable on the
    array (similar_message_environment, messagecache.jl:205-229)."""
    out = {}
    for u, v in _all_edges(nn.ket):
        ket = nn.ket.linknames(u, v)
        dims = [_dim_of(nn.ket[u], n) for n in ket]
        D = int(np.prod(dims))
        if f == "one":
            mat = np.eye(D)
        elif f == "ones":
            mat = np.ones((D, D))
        else:
            mat = np.asarray(f(np.zeros((D, D))))
        bra_inds = [Index(d, nn.bra(n)) for d, n in zip(dims, ket)]
        ket_inds = [Index(d, n) for d, n in zip(dims, ket)]
        dt = nn.ket[u].data.dtype
        out[(u, v)] = ITensor(mat.astype(np.result_type(dt, mat.dtype)).reshape(dims + dims),
                              bra_inds + ket_inds)
    return MessageCache(out)


def _dim_of(t: ITensor, name):
    return t.inds[t.dimnames.index(name)].dim


def _all_edges(tn: ITensorNetwork):
    out = []
    for u, v in tn.edges():
        out += [(u, v), (v, u)]
    return out


# ---- flattening onto the C ABI -------------------------------------------------------------------
class _Flat:
    """CSR graph + canonical packed tensors of a network, with the slot of every directed
    edge and the (bra, ket) or (link) names of every message."""

    def __init__(self, factors):
        self.norm = isinstance(factors, NormNetwork)
        tn = factors.ket if self.norm else factors
        self.tn = tn
        self.vs = tn.vertices()
        self.vidx = {v: k for k, v in enumerate(self.vs)}
        edges, bonds, self.linkgroups = [], [], {}
        for u, v in tn.edges():
            names = tn.linknames(u, v)
            edges.append((self.vidx[u], self.vidx[v]))
            bonds.append(int(np.prod([_dim_of(tn[u], n) for n in names])))
            self.linkgroups[(u, v)] = names
            self.linkgroups[(v, u)] = names
        phys = []
        for v in self.vs:
            sites = tn.sitenames(v)
            phys.append(int(np.prod([_dim_of(tn[v], n) for n in sites])) if sites else 1)
        if not self.norm and any(p != 1 for p in phys):
            raise ItnArgumentError(1, "belief propagation on a plain network needs tensors without open site indices")
        self.g = G.from_edges(len(self.vs), edges, bonds, phys=phys, layers=2 if self.norm else 1)
        self.slot = {}
        for k, v in enumerate(self.vs):
            for s in range(self.g.off[k], self.g.off[k + 1]):
                self.slot[(v, self.vs[int(self.g.nbr[s])])] = int(s)
        dt = np.result_type(*[tn[v].data.dtype for v in self.vs])
        self.dtype = np.dtype(np.complex128) if dt.kind == "c" else np.dtype(np.float64)
        packed = np.zeros(int(self.g.toff[-1]), dtype=self.dtype)
        for k, v in enumerate(self.vs):
            order = list(tn.sitenames(v))
            for s in range(self.g.off[k], self.g.off[k + 1]):
                order += self.linkgroups[(v, self.vs[int(self.g.nbr[s])])]
            packed[self.g.toff[k]:self.g.toff[k + 1]] = tn[v].permute(order).ravel()
        self.tensors = packed

    def pack_messages(self, cache: MessageCache, nn=None):
        m = np.zeros(int(self.g.moff[-1]), dtype=self.dtype)
        for (u, v), s in self.slot.items():
            ket = self.linkgroups[(u, v)]
            t = cache[(u, v)]
            if self.norm:
                bra = [nn.bra(n) for n in ket]
                block = t.permute(bra + ket)
            else:
                block = t.permute(ket)
            m[self.g.moff[s]:self.g.moff[s + 1]] = block.ravel()
        return m

    def unpack_messages(self, m, like: MessageCache, nn=None):
        out = {}
        for (u, v), s in self.slot.items():
            ket = self.linkgroups[(u, v)]
            t = like[(u, v)]
            blk = m[self.g.moff[s]:self.g.moff[s + 1]]
            if self.norm:
                bra = [nn.bra(n) for n in ket]
                names = bra + ket
            else:
                names = ket
            dims = [_dim_of(t, n) for n in names]
            arr = blk.reshape(dims)
            # back to the message's own index order
            perm = [names.index(n) for n in t.dimnames]
            out[(u, v)] = ITensor(np.transpose(arr, perm), t.inds)
        return MessageCache(out)

    def engine(self, cache=None, nn=None):
        e = BPEngine(self.g)
        e.set_tensors(self.tensors)
        if cache is not None:
            e.set_messages(self.pack_messages(cache, nn))
        return e


# ---- algorithms --------------------------------------------------------------------------------
@dataclass
class Exact:
    """contract_network's exact algorithm (contract_network.jl:7-10); order_alg is Greedy()
    (the default), LeftAssociative(), Sweep() or the strings "greedy" / "left" / "sweep"."""
    order: object = None
    order_alg: str = "greedy"


class Greedy:
    pass


class LeftAssociative:
    pass


class Sweep:
    """Order algorithm of this library (no counterpart in the reference): the cheaper, in
    multiply-adds, of the greedy order and running-product orders that absorb at every step the
    tensor leaving the product smallest -- boundary sweeps on lattices."""


@dataclass
class SimpleMessageUpdate:
    """The reference's message update (beliefpropagation.jl:237-240): sequential sweep over
    ``edges``, normalised by the sum of entries."""
    normalize: bool = True
    contraction_alg: Exact = field(default_factory=Exact)


@dataclass
class GPUMessageUpdate:
    """Whole-solve GPU strategy: ``schedule`` "parallel" (Jacobi) or "sequential";
    ``precision`` "native", or "bf16" / "tf32" / "tf32x3" (tcgen05; float32 norm networks
    with at most 4 legs per vertex, bonds of at most 8 and d <= 2, smaller vertices
    zero-padded to 4 legs of 8 and d = 2) with ``split_sweeps`` final split-precision
    sweeps."""
    normalize: bool = True
    schedule: str = "parallel"
    precision: str = "native"
    split_sweeps: int = 0


@dataclass
class StopAfterIteration:
    maxiter: int


@dataclass
class StopWhenConverged:
    tol: float


class StopWhenAny:
    def __init__(self, *cs):
        self.criteria = cs


def select_beliefpropagation_stopping_criterion(c):
    """(beliefpropagation.jl:16-55): a NamedTuple-like dict with maxiter and/or tol, or
    criterion objects; raises ArgumentError-equivalents otherwise."""
    if c is None:
        raise ItnArgumentError(1, "`stopping_criterion` must be specified, e.g. "
                                  "`stopping_criterion = (; maxiter = 10)`")
    if isinstance(c, StopAfterIteration):
        return c.maxiter, None
    if isinstance(c, StopWhenConverged):
        return None, c.tol
    if isinstance(c, StopWhenAny):
        mi, tol = None, None
        for x in c.criteria:
            a, b = select_beliefpropagation_stopping_criterion(x)
            mi = a if a is not None else mi
            tol = b if b is not None else tol
        return mi, tol
    if isinstance(c, dict):
        extra = set(c) - {"maxiter", "tol"}
        if extra:
            raise ItnArgumentError(1, f"Unrecognized `stopping_criterion` kwargs: {tuple(sorted(extra))}. "
                                      "Supported: `maxiter`, `tol`.")
        mi, tol = c.get("maxiter"), c.get("tol")
        if mi is None and tol is None:
            raise ItnArgumentError(1, "At least one of `maxiter` or `tol` must be specified.")
        return mi, tol
    raise ItnArgumentError(1, f"unsupported stopping criterion {c!r}")


def default_beliefpropagation_edges(flat: _Flat):
    """Sweep order when none is given: leaves-to-root then root-to-leaves over a spanning
    forest, then the remaining edges both ways (the role of forest_cover_edge_sequence)."""
    return [(flat.vs[flat.g.slot_src(int(s))], flat.vs[int(flat.g.nbr[int(s)])])
            for s in G.tree_edge_sequence(flat.g)]


def beliefpropagation(factors, messages, *, edges=None, stopping_criterion=None,
                      message_update_algorithm=None):
    """beliefpropagation(factors, messages; edges, stopping_criterion, message_update_algorithm)
    -> MessageCache (beliefpropagation.jl:69-92), solved on the GPU."""
    maxiter, tol = select_beliefpropagation_stopping_criterion(stopping_criterion)
    alg = message_update_algorithm or SimpleMessageUpdate()
    if isinstance(alg, dict):
        alg = SimpleMessageUpdate(**alg)
    cache = messages if isinstance(messages, MessageCache) else MessageCache(messages)
    flat = _Flat(factors)
    nn = factors if flat.norm else None
    sched = "sequential" if isinstance(alg, SimpleMessageUpdate) else alg.schedule
    kw = {}
    if isinstance(alg, GPUMessageUpdate) and alg.precision != "native":
        kw = dict(precision=alg.precision, split_sweeps=alg.split_sweeps)
    tens = flat.tensors
    if kw:
        tens = tens.astype(np.float32)
    e = BPEngine(flat.g)
    try:
        e.set_tensors(tens)
        e.set_messages(flat.pack_messages(cache, nn).astype(tens.dtype))
        ed = None
        if sched == "sequential":
            es = edges if edges is not None else default_beliefpropagation_edges(flat)
            ed = np.asarray([flat.slot[tuple(x)] for x in es], dtype=np.int64)
        e.run(schedule=sched, edges=ed, maxiter=maxiter, tol=tol, normalize=alg.normalize, **kw)
        m = e.messages().astype(flat.dtype)
    finally:
        e.close()
    return flat.unpack_messages(m, cache, nn)


def message_update(cache: MessageCache, factors, edge, alg=None):
    """message_update!(alg, cache, factors, edge) (beliefpropagation.jl:242-257), in place
    on ``cache``; returns it."""
    alg = alg or SimpleMessageUpdate()
    flat = _Flat(factors)
    nn = factors if flat.norm else None
    with flat.engine(cache, nn) as e:
        e.message_update(flat.slot[tuple(edge)], normalize=alg.normalize)
        new = flat.unpack_messages(e.messages(), cache, nn)
    cache[tuple(edge)] = new[tuple(edge)]
    return cache


def iterate_diff(cache1: MessageCache, cache2: MessageCache):
    """max over directed edges of 1 - |<m1/|m1|, m2/|m2|>|^2 (beliefpropagation.jl:261-267),
    FP64 on the device.  Each message becomes one two-vertex component whose single edge
    carries it (both directions hold the same vector, which leaves the maximum unchanged)."""
    edges = cache1.edges()
    a = [np.asarray(cache1[e].data).ravel() for e in edges]
    b = [np.asarray(cache2[e].permute(cache1[e].dimnames)).ravel() for e in edges]
    dt = np.result_type(*[x.dtype for x in a + b], np.float64)
    comps = [G.from_edges(2, [(0, 1)], [x.size], phys=1, layers=1) for x in a]
    g = G.batched(comps)
    aa = np.concatenate([np.concatenate([x, x]) for x in a]).astype(dt)
    bb = np.concatenate([np.concatenate([y, y]) for y in b]).astype(dt)
    with BPEngine(g) as e:
        e.set_tensors(np.ones(int(g.toff[-1]), dtype=dt))
        return e.iterate_diff(aa, bb)


def _scalars(factors, messages):
    flat = _Flat(factors)
    nn = factors if flat.norm else None
    with flat.engine(messages, nn) as e:
        r = e.logscalars()
    return flat, r


def vertex_scalars(factors, messages, vertices=None):
    flat, r = _scalars(factors, messages)
    vs = vertices if vertices is not None else flat.vs
    return [r["zv"][flat.vidx[v]] for v in vs]


def vertex_scalar(factors, messages, vertex):
    """Full contraction of the factor of ``vertex`` with all its incoming messages
    (messagecache.jl:139-143)."""
    return vertex_scalars(factors, messages, [vertex])[0]


def edge_scalar(cache: MessageCache, edge):
    """edge_scalar(cache, edge) (messagecache.jl:153-157): contract_network of the two
    messages of an edge, m(u->v) and m(v->u), over all their shared names."""
    return edge_scalars(cache, [tuple(edge)])[0]


def edge_scalars(cache: MessageCache, edges=None):
    """edge_scalars(cache[, edges]) (messagecache.jl:159-178): one scalar per edge of
    ``edges`` (default: every edge of the cache), skipping repeats and reverses, in order.
    All pairs are contracted in one device call: each pair becomes a two-vertex component
    whose messages are the flattened pair, so its edge scalar is their full contraction."""
    edges = [tuple(e) for e in (cache.keys() if edges is None else edges)]
    seen, keep = set(), []
    for e in edges:
        r = (e[1], e[0])
        if e in seen or r in seen:
            continue
        seen.add(e)
        keep.append(e)
    if not keep:
        return []
    a = [np.asarray(cache[e].data).ravel() for e in keep]
    b = [np.asarray(cache[(e[1], e[0])].permute(cache[e].dimnames)).ravel() for e in keep]
    dt = np.result_type(*[x.dtype for x in a + b], np.float64)
    g = G.batched([G.from_edges(2, [(0, 1)], [x.size], phys=1, layers=1) for x in a])
    mm = np.concatenate([np.concatenate([x, y]) for x, y in zip(a, b)]).astype(dt)
    with BPEngine(g) as e:
        e.set_tensors(np.ones(int(g.toff[-1]), dtype=dt))
        e.set_messages(mm)
        ze = e.logscalars()["ze"]
    return list(ze)


def region_scalar(factors, messages, region):
    return np.prod(vertex_scalars(factors, messages, list(region)))


def bethe_free_energy(factors, messages):
    """sum log Z_v - sum log Z_e with the reference's promotion rules
    (messagecache.jl:185-201), FP64 log-scalars on the device."""
    flat = _Flat(factors)
    nn = factors if flat.norm else None
    with flat.engine(messages, nn) as e:
        return e.bethe_free_energy()


def contract_network(tn, alg=None):
    """contract_network(tn; alg = Exact()) (contract_network.jl:12-37): tn is a list of
    ITensors, an ITensorNetwork or a NormNetwork.  Returns an ITensor."""
    alg = alg if alg is not None else Exact()
    if not isinstance(alg, Exact):
        raise ItnArgumentError(1, f"`contract_network` algorithm `{alg}` not implemented.")
    if isinstance(tn, NormNetwork):
        ts = []
        for v in tn.vertices():
            ts += [tn.kettensor(v), tn.conj_bratensor(v).conj()]
    elif isinstance(tn, ITensorNetwork):
        ts = [tn[v] for v in tn.vertices()]
    else:
        ts = list(tn)
    order_alg = alg.order_alg
    if isinstance(order_alg, Greedy):
        order_alg = "greedy"
    elif isinstance(order_alg, LeftAssociative):
        order_alg = "left"
    elif isinstance(order_alg, Sweep):
        order_alg = "sweep"
    kw = dict(alg=order_alg) if alg.order is None else dict(steps=alg.order)
    data, labels = _contract_arrays([t.data for t in ts], [list(t.dimnames) for t in ts], **kw)
    dims = {}
    for t in ts:
        for i in t.inds:
            dims[i.name] = i.dim
    return ITensor(data, [Index(dims[n], n) for n in labels])


# ---- gate application (src/apply/apply_operators.jl) -------------------------------------------
class Operator(ITensor):
    """A named operator (ITensorBase ``operator(data, codomain, domain)``): data with axes
    (codomain..., domain...); applying it contracts the domain names with a tensor and
    renames the codomain back to the domain names."""

    def __init__(self, data, codomain_inds, domain_inds):
        super().__init__(data, list(codomain_inds) + list(domain_inds))
        self.codomain = tuple(i.name for i in codomain_inds)
        self.domain = tuple(i.name for i in domain_inds)


def operator(data, codomain_inds, domain_inds):
    return Operator(data, codomain_inds, domain_inds)


@dataclass
class BPApplyGate:
    """Default single-operator strategy (apply_operators.jl:190-224): BP simple update.
    ``trunc`` = max rank (int), (max_rank, cutoff) or None; ``normalize`` rescales
    (the singular values of a two-site gate to unit norm, a one-site result to unit
    gauged norm)."""
    trunc: object = None
    normalize: bool = False


def _trunc_args(trunc):
    if trunc is None:
        return None, None
    if isinstance(trunc, (tuple, list)):
        return trunc[0], trunc[1]
    return int(trunc), None


def operator_message_cache(nn: NormNetwork, messages: MessageCache):
    """BP messages (bra and ket link indices) as operators with codomain = bra names and
    domain = ket names: the environment format apply_operator consumes
    (test/test_apply_operator.jl:42-53; message_environment, messagecache.jl:205-229)."""
    out = {}
    for (u, v) in messages.keys():
        t = messages[(u, v)]
        ket = nn.ket.linknames(u, v)
        bra = [nn.bra(n) for n in ket]
        dims = {i.name: i.dim for i in t.inds}
        data = t.permute(bra + ket)
        out[(u, v)] = Operator(data, [Index(dims[n], n) for n in bra], [Index(dims[n], n) for n in ket])
    return MessageCache(out)


def _env_matrix(env: MessageCache, edge, ket_names):
    """The D x D matrix M[bra, ket] of env[edge], ket axes in the order of ket_names."""
    t = env[edge]
    if isinstance(t, Operator):
        # codomain (bra) x domain (ket), domain matched to ket_names by position
        pair = dict(zip(t.domain, t.codomain))
        if set(pair) != set(ket_names):
            raise ItnArgumentError(1, f"environment of {edge} does not carry the link names")
        arr = t.permute([pair[n] for n in ket_names] + list(ket_names))
        D = int(np.prod([_dim_of(t, n) for n in ket_names]))
        return arr.reshape(D, D)
    k = len(t.inds) // 2
    bra, ket = list(t.dimnames[:k]), list(t.dimnames[k:])
    if set(ket) != set(ket_names):
        # the bra names may come first or second: find the half that holds the link names
        bra, ket = ket, bra
        if set(ket) != set(ket_names):
            raise ItnArgumentError(1, f"environment of {edge} does not carry the link names")
    pair = {kn: bn for kn, bn in zip(ket, bra)}
    order = [pair[n] for n in ket_names] + list(ket_names)
    arr = t.permute(order)
    D = int(np.prod([_dim_of(t, n) for n in ket_names]))
    return arr.reshape(D, D)


def _gate_site(state: ITensorNetwork, v, domain, partner, env):
    """Site array [other legs..., s(, b)] of vertex v for a gate with the given domain names,
    the names of each axis group and the environments of the gauged legs."""
    t = state[v]
    groups, envs = [], []
    for w in state.neighbors(v):
        if w == partner:
            continue
        names = state.linknames(v, w)
        groups.append(names)
        envs.append(_env_matrix(env, (w, v), names) if env is not None and (w, v) in env.keys() else None)
    extra = [n for n in state.sitenames(v) if n not in domain]
    for n in extra:
        groups.append([n])
        envs.append(None)
    mine = [n for n in domain if n in t.dimnames]
    bond = state.linknames(v, partner) if partner is not None else []
    order = [n for g in groups for n in g] + mine + bond
    shape = [int(np.prod([_dim_of(t, n) for n in g])) for g in groups]
    shape += [int(np.prod([_dim_of(t, n) for n in mine]))]
    if partner is not None:
        shape += [int(np.prod([_dim_of(t, n) for n in bond]))]
    return t.permute(order).reshape(shape), groups, mine, envs


def _op_matrix(op: Operator, domains):
    """op as [s1', (s2',) s1, (s2)] with each s the fused names of one site's domain part."""
    cod_of = dict(zip(op.domain, op.codomain))
    order = [cod_of[n] for d in domains for n in d] + [n for d in domains for n in d]
    arr = op.permute(order)
    dims = [int(np.prod([_dim_of(op, n) for n in d])) for d in domains]
    return arr.reshape(dims + dims)


def _gate_vertices(op: Operator, state: ITensorNetwork):
    vs = [v for v in state.vertices() if set(op.domain) & set(state.sitenames(v))]
    if not vs:
        raise ItnArgumentError(1, "operator shares no indices with the tensor network")
    if len(vs) > 2:
        raise ItnArgumentError(1, f"{len(vs)}-site gate decomposition not implemented")
    return vs


def _gate_of(op: Operator, state: ITensorNetwork, env: MessageCache):
    from .apply import Gate
    vs = _gate_vertices(op, state)
    if len(vs) == 1:
        v = vs[0]
        psi, groups, mine, envs = _gate_site(state, v, op.domain, None, env)
        return Gate([psi], [envs], _op_matrix(op, [mine]), extra=dict(vs=vs, groups=[groups], mine=[mine]))
    v1, v2 = vs
    if not state.linknames(v1, v2):
        raise ItnArgumentError(1, "a two-site gate needs neighbouring vertices")
    p1, g1, m1, e1 = _gate_site(state, v1, op.domain, v2, env)
    p2, g2, m2, e2 = _gate_site(state, v2, op.domain, v1, env)
    return Gate([p1, p2], [e1, e2], _op_matrix(op, [m1, m2]), extra=dict(vs=vs, groups=[g1, g2], mine=[m1, m2]))


def _finish(state: ITensorNetwork, env: MessageCache, gate, result):
    dest = dict(state.tensors)
    env2 = env.copy() if env is not None else MessageCache({})
    vs = gate.extra["vs"]
    if len(vs) == 1:
        v = vs[0]
        t = state[v]
        groups, mine = gate.extra["groups"][0], gate.extra["mine"][0]
        names = [n for g in groups for n in g] + mine
        arr = result.reshape([_dim_of(t, n) for n in names])
        dest[v] = ITensor(arr, [Index(_dim_of(t, n), n) for n in names])
        return ITensorNetwork(dest), env2
    n1, n2, S = result
    chi = len(S)
    bond = Index(chi, uniquename())
    for i, (v, arr) in enumerate(zip(vs, (n1, n2))):
        t = state[v]
        groups, mine = gate.extra["groups"][i], gate.extra["mine"][i]
        names = [n for g in groups for n in g] + mine
        a = arr.reshape([_dim_of(t, n) for n in names] + [chi])
        dest[v] = ITensor(a, [Index(_dim_of(t, n), n) for n in names] + [bond])
    v1, v2 = vs
    dt = np.result_type(n1.dtype, np.float64) if n1.dtype.kind != "c" else n1.dtype
    diag = np.diag(S).astype(dt)
    env2[(v1, v2)] = ITensor(diag, [Index(chi, uniquename()), bond])
    env2[(v2, v1)] = ITensor(diag.copy(), [Index(chi, uniquename()), bond])
    return ITensorNetwork(dest), env2


def apply_operator(op: Operator, state: ITensorNetwork, env: MessageCache, *, alg=None, trunc=None,
                   normalize=None, context=None):
    """apply_operator(operator, state, env; alg, kwargs...) -> (state, env)
    (apply_operators.jl:147-188, BP simple update :226-283), on the GPU."""
    return apply_operators([op], state, env, alg=alg, trunc=trunc, normalize=normalize, context=context)


def apply_operators(ops, state: ITensorNetwork, env: MessageCache, *, alg=None, trunc=None, normalize=None,
                    context=None):
    """apply_operators(operators, state, env; alg, kwargs...) -> (state, env)
    (apply_operators.jl:14-120): the operators in turn, each updating the state and the
    environment of its bond.  Consecutive operators on disjoint vertices are applied in
    one GPU batch (the result is the same as one by one: each gate reads only its own
    sites and the environments of edges into them; another gate changes only its own
    sites and the environments of its own bond)."""
    from .apply import apply_gates
    alg = alg if alg is not None else BPApplyGate()
    if trunc is not None:
        alg = BPApplyGate(trunc=trunc, normalize=alg.normalize)
    if normalize is not None:
        alg = BPApplyGate(trunc=alg.trunc, normalize=bool(normalize))
    max_rank, cutoff = _trunc_args(alg.trunc)
    ops = list(ops)
    if not ops:
        return ITensorNetwork(dict(state.tensors)), (env.copy() if env is not None else None)
    k = 0
    while k < len(ops):
        # the longest run of operators on pairwise disjoint vertices
        batch, used = [], set()
        while k < len(ops):
            vs = _gate_vertices(ops[k], state)
            touch = set(vs)
            if batch and touch & used:
                break
            batch.append(_gate_of(ops[k], state, env))
            used |= touch
            k += 1
        results = apply_gates(batch, max_rank=max_rank, cutoff=cutoff, normalize=alg.normalize, context=context)
        for gate, res in zip(batch, results):
            state, env = _finish(state, env, gate, res)
    return state, env
