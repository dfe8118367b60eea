"""The single sweep split along the lattice's last axis into column slabs, one per rank.

ArrayBackend threads its sweep by contiguous slabs of the last axis (src/backends.jl:457-479):
every thread updates its own columns from one shared, halo-padded array. Here the ranks share no
memory. Each rank holds its slab plus h columns of halo on each side where the lattice goes on,
runs K steps on that padded slab with the library's kernels, and then trades h columns with each
neighbour: its first owned columns to the left, its last to the right, with periodic wrap at the
ends of a torus. A step reads neighbours at most r columns away (2r for Checkerboard's two
half-sweeps), so after K steps only the h = r K gates outermost columns can have read a wrong
value, and the owned columns are exact. gbca_set_slab gives the slab its global cell ids and
Checkerboard parities, so every draw is the one the whole lattice makes.

Summaries add up exactly: each rank sums its owned cells' integers (gbca_slab_sums: value
counts, and Moran's I's S, S2, P, Q, W), one all-reduce adds the ranks', and Moran's I is
finished as the exact ratio of src/measures.jl:91-107.

Transports: ProcessGroupTransport over torch.distributed (NCCL between GPUs, gloo on the CPU)
and LocalGroup, which runs several slabs in one process (one GPU, one slab after another)."""
from __future__ import annotations

import ctypes
import contextlib
from dataclasses import dataclass
from fractions import Fraction
from typing import List, Optional, Sequence

import numpy as np

from . import capi
from .errors import ArgumentError, UnsupportedCombinationError
from .model import Checkerboard, KernelSI, Lenia, Periodic

SUMS = 261  # gbca_slab_sums: 256 value counts, then S, S2, P, Q, W


@dataclass(frozen=True)
class Slab:
    """One rank's share: owned global columns [j0, j1), halo columns held on each side (lpad,
    rpad) and the neighbours that send them (None at an edge of a lattice that does not wrap)."""
    rank: int
    world: int
    j0: int
    j1: int
    lpad: int
    rpad: int
    left: Optional[int]
    right: Optional[int]

    @property
    def own(self) -> int:
        return self.j1 - self.j0

    @property
    def width(self) -> int:
        return self.own + self.lpad + self.rpad

    @property
    def col0(self) -> int:
        """Global column of the padded slab's first column (negative on a torus's first rank)."""
        return self.j0 - self.lpad


def slab_bounds(n2: int, world: int) -> List[tuple]:
    """Owned columns of each rank: contiguous, as equal as possible, the first n2 mod world
    ranks one column more."""
    if world < 1 or n2 < world:
        raise ArgumentError(f"{n2} columns cannot be split among {world} ranks")
    base, extra = divmod(n2, world)
    out, j = [], 0
    for r in range(world):
        k = base + (1 if r < extra else 0)
        out.append((j, j + k))
        j += k
    return out


def halo_columns(radius: int, steps_per_exchange: int, gates: int = 1) -> int:
    """Columns a slab must hold on each side to run steps_per_exchange steps between exchanges:
    radius per sweep, gates sweeps per step (2 for Checkerboard)."""
    return radius * steps_per_exchange * gates


def plan(n2: int, world: int, h: int, periodic: bool) -> List[Slab]:
    """The slabs of an n2-column lattice on `world` ranks with h halo columns. Every slab owns at
    least h columns (a halo then comes from one neighbour) and no padded slab is wider than the
    lattice."""
    bounds = slab_bounds(n2, world)
    if world == 1:
        return [Slab(0, 1, 0, n2, 0, 0, None, None)]
    slabs = []
    for r, (j0, j1) in enumerate(bounds):
        if j1 - j0 < h:
            raise ArgumentError(f"rank {r} would own {j1 - j0} columns, fewer than the {h}-column halo: "
                                "use fewer ranks or fewer steps between exchanges")
        if periodic:
            left, right, lp, rp = (r - 1) % world, (r + 1) % world, h, h
        else:
            left = r - 1 if r > 0 else None
            right = r + 1 if r < world - 1 else None
            lp, rp = (h if left is not None else 0), (h if right is not None else 0)
        s = Slab(r, world, j0, j1, lp, rp, left, right)
        if s.width > n2:
            raise ArgumentError(f"rank {r}'s padded slab ({s.width} columns) is wider than the lattice ({n2})")
        slabs.append(s)
    return slabs


def exchange_ops(s: Slab):
    """The point-to-point messages of one halo exchange, in the order every rank posts them:
    last owned columns to the right neighbour, left halo from the left one, first owned columns to
    the left neighbour, right halo from the right one. Between any two ranks (two on a torus of
    two ranks) the sends of one and the receives of the other then pair up in posting order,
    which is how NCCL matches them. Each op: (kind, peer, tag, first column, column count)."""
    h_l, h_r, own = s.lpad, s.rpad, s.own
    ops = []
    if s.right is not None:
        ops.append(("send", s.right, 0, h_l + own - h_r, h_r))
    if s.left is not None:
        ops.append(("recv", s.left, 0, 0, h_l))
    if s.left is not None:
        ops.append(("send", s.left, 1, h_l, h_l))
    if s.right is not None:
        ops.append(("recv", s.right, 1, h_l + own, h_r))
    return ops


def morans_from_sums(sums: Sequence[int], n: int) -> float:
    """Moran's I from the integer sums S, S2, P, Q, W over n cells (NaN for a constant field):
    (n^2 P - n S Q + W S^2) / (W (n S2 - S^2)), computed exactly and rounded once."""
    S, S2, P, Q, W = (int(x) for x in sums)
    num = n * n * P - n * S * Q + W * S * S
    den = W * (n * S2 - S * S)
    if den == 0 or W == 0:
        return float("nan")
    return float(Fraction(num, den))


def summaries_from_sums(total: Sequence[int], n: int, nvals: int = 3):
    """(counts[0:nvals], cells outside 0..nvals-1, Moran's I) from a lattice's summed sums."""
    hist = [int(x) for x in total[:256]]
    counts = [hist[v + 128] for v in range(nvals)]
    return counts, n - sum(counts), morans_from_sums(total[256:261], n)


def _check_problem(prob, scheme):
    if isinstance(prob.rule, (Lenia, KernelSI)) or getattr(prob, "fields", None):
        raise UnsupportedCombinationError("slabs run rules without kernel fields (Life, Generations, forest fire)")
    if getattr(prob, "covariates", None):
        raise UnsupportedCombinationError("slabs run problems without covariates")


def gates_of(scheme) -> int:
    return 2 if isinstance(scheme, Checkerboard) else 1


class _DevColumns:
    """A run of whole columns of a device state as a CUDA array (for torch.as_tensor)."""

    def __init__(self, ptr: int, ncols: int, pitch: int):
        self.__cuda_array_interface__ = {"shape": (ncols, pitch), "typestr": "|i1", "data": (ptr, False),
                                         "version": 3, "strides": None, "stream": None}


class DeviceSlab:
    """A padded slab on this process's GPU: a libgbca handle of n1 x width cells, placed in the
    lattice with gbca_set_slab. Its sweeps run on `stream` (a torch.cuda.Stream; a new one if
    None), and the halo copies and collectives run on the same stream (context()), so each is
    ordered after the sweep it reads and before the sweep that reads it."""

    def __init__(self, prob, scheme, slab: Slab, u=None, stream=None):
        import torch

        from .backend import make_desc
        _check_problem(prob, scheme)
        n1, n2 = prob.space.dims
        self.slab, self.n1, self.n2 = slab, n1, n2
        d = make_desc(prob, scheme)
        d.n2 = slab.width
        self.cols = (slab.col0 + np.arange(slab.width)) % n2
        self.handle = ctypes.c_void_p()
        lib = capi.lib()
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(self.handle)))
        self.torch = torch
        self.stream = stream if stream is not None else torch.cuda.Stream()
        capi.check(lib.gbca_set_stream(self.handle, ctypes.c_void_p(self.stream.cuda_stream)))
        capi.check(lib.gbca_set_slab(self.handle, slab.col0, n2))
        if prob.mask is not None:
            m = np.asfortranarray(np.asarray(prob.mask, dtype=np.uint8)[:, self.cols])
            capi.check(lib.gbca_set_mask(self.handle, m.ctypes.data, m.nbytes))
        self.set_global(np.asarray(prob.u0) if u is None else u)

    def set_global(self, u):
        """The slab's columns (halo included) of a whole-lattice state."""
        a = np.asfortranarray(np.asarray(u, dtype=np.int8)[:, self.cols])
        capi.check(capi.lib().gbca_set_state(self.handle, a.ctypes.data, a.nbytes))

    def context(self):
        """Work queued inside runs on the slab's stream."""
        return self.torch.cuda.stream(self.stream)

    def set_state_device(self, cols) -> None:
        """The padded slab's state from a device tensor holding its width columns of n1 bytes
        (contiguous), queued on the slab's stream."""
        capi.check(capi.lib().gbca_set_state_device(self.handle, ctypes.c_void_p(cols.data_ptr()), self.n1))

    def step(self, t: int, k: int, params) -> None:
        vals = tuple(params or ())
        arr = (ctypes.c_double * max(1, len(vals)))(*vals)
        capi.check(capi.lib().gbca_advance(self.handle, int(t), int(k), arr, len(vals)))

    def columns(self, a: int, k: int):
        """Columns a .. a + k - 1 of the current state as an int8 device tensor (k x pitch bytes;
        a column's bytes past n1 travel along unread)."""
        ptr, pitch = ctypes.c_void_p(), ctypes.c_int64()
        capi.check(capi.lib().gbca_device_state(self.handle, ctypes.byref(ptr), ctypes.byref(pitch)))
        return self.torch.as_tensor(_DevColumns(ptr.value + a * pitch.value, k, pitch.value), device="cuda")

    def read(self) -> np.ndarray:
        out = np.empty((self.n1, self.slab.width), np.int8, order="F")
        capi.check(capi.lib().gbca_get_state(self.handle, out.ctypes.data, out.nbytes))
        return out

    def sums(self, j_lo: int, j_hi: int) -> np.ndarray:
        out = np.zeros(SUMS, np.int64)
        capi.check(capi.lib().gbca_slab_sums(self.handle, int(j_lo), int(j_hi),
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    def close(self):
        if self.handle:
            capi.lib().gbca_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _context(shard):
    ctx = getattr(shard, "context", None)
    return ctx() if ctx else contextlib.nullcontext()


class ProcessGroupTransport:
    """Halo exchange and sums over torch.distributed: NCCL with device slabs, gloo with host
    ones. Sends and receives of one exchange go out as one batch (batch_isend_irecv). A gloo
    group with device slabs (gloo moves host memory only) stages the columns through host
    memory: the sent ones copied out first, the received ones copied in after the batch."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist, self.group = dist, group
        self.host_staged = dist.get_backend(group) == "gloo"

    def exchange(self, shard, ops) -> None:
        dist = self.dist
        with _context(shard):
            p2p, landing = [], []
            for kind, peer, tag, a, k in ops:
                if k == 0:
                    continue
                cols = shard.columns(a, k)
                if self.host_staged and cols.is_cuda:
                    host = cols.cpu() if kind == "send" else cols.new_empty(cols.shape, device="cpu")
                    if kind == "recv":
                        landing.append((cols, host))
                    cols = host
                fn = dist.isend if kind == "send" else dist.irecv
                p2p.append(dist.P2POp(fn, cols, peer, self.group, tag))
            if p2p:
                for req in dist.batch_isend_irecv(p2p):
                    req.wait()
            for cols, host in landing:
                cols.copy_(host)

    def allreduce_sums(self, local: np.ndarray, device) -> np.ndarray:
        import torch
        t = torch.as_tensor(local, dtype=torch.int64, device=device)
        self.dist.all_reduce(t, group=self.group)
        return t.cpu().numpy()

    def gather_owned(self, block: np.ndarray, slab: Slab, n2: int, root: int = 0, device="cpu"):
        """The whole lattice on `root` from every rank's owned columns; None elsewhere."""
        import torch
        dist = self.dist
        n1 = block.shape[0]
        if slab.rank == root:
            out = np.empty((n1, n2), np.int8, order="F")
            out[:, slab.j0:slab.j1] = block
            for r, (j0, j1) in enumerate(slab_bounds(n2, slab.world)):
                if r == root:
                    continue
                buf = torch.empty((j1 - j0, n1), dtype=torch.int8, device=device)
                dist.recv(buf, src=r, group=self.group)
                out[:, j0:j1] = buf.cpu().numpy().T
            return out
        dist.send(torch.as_tensor(np.ascontiguousarray(block.T), device=device), dst=root, group=self.group)
        return None


class SlabSweep:
    """One rank's part of a sharded single sweep: `shard` holds the padded slab (a DeviceSlab, or
    any object with step / columns / read / sums), `transport` exchanges halos and adds sums."""

    def __init__(self, prob, scheme, slab: Slab, shard, transport, steps_per_exchange: int):
        _check_problem(prob, scheme)
        self.prob, self.slab, self.shard, self.transport = prob, slab, shard, transport
        self.K = int(steps_per_exchange)
        self.h = halo_columns(prob.neighbours.radius, self.K, gates_of(scheme))
        if slab.world > 1 and (slab.lpad not in (0, self.h) or slab.rpad not in (0, self.h)):
            raise ArgumentError(f"the slab's halo ({slab.lpad}, {slab.rpad}) is not the {self.h} columns that "
                                f"{self.K} steps between exchanges need")
        self.ops = exchange_ops(slab)

    def exchange(self) -> None:
        self.transport.exchange(self.shard, self.ops)

    def run(self, t0: int, nsteps: int, params=None) -> None:
        """Steps t0 .. t0 + nsteps - 1: an exchange, then up to K steps on the padded slab."""
        t = int(t0)
        while nsteps > 0:
            k = min(self.K, nsteps)
            if self.slab.world > 1:
                self.exchange()
            self.shard.step(t, k, params)
            t += k
            nsteps -= k

    def owned(self) -> np.ndarray:
        s = self.slab
        return np.asfortranarray(self.shard.read()[:, s.lpad:s.lpad + s.own])

    def summaries(self, nvals: int = 3, device="cpu"):
        """Counts and Moran's I of the whole lattice (every rank gets them): halos refreshed, owned
        cells summed on each rank, one all-reduce."""
        if self.slab.world > 1:
            self.exchange()
        s = self.slab
        local = self.shard.sums(s.lpad, s.lpad + s.own)
        total = self.transport.allreduce_sums(local, device) if s.world > 1 else local
        n1, n2 = self.prob.space.dims
        return summaries_from_sums(total, n1 * n2, nvals)


class LocalGroup:
    """Every slab of a lattice in one process, exchanged by direct copies: the sharded sweep on
    one GPU (or, with host shards, on the CPU), one slab after another. No slab waits on another
    inside a kernel; the exchanges sit between passes."""

    def __init__(self, prob, scheme, world: int, steps_per_exchange: int, make_shard=None):
        _check_problem(prob, scheme)
        n1, n2 = prob.space.dims
        self.prob, self.K = prob, int(steps_per_exchange)
        self.h = halo_columns(prob.neighbours.radius, self.K, gates_of(scheme))
        periodic = isinstance(prob.space.boundaries[1], Periodic)
        self.slabs = plan(n2, world, self.h, periodic)
        if make_shard is None:  # device slabs, all on one stream: sweeps and copies in issue order
            import torch
            stream = torch.cuda.Stream()
            make_shard = lambda s: DeviceSlab(prob, scheme, s, stream=stream)  # noqa: E731
        self.shards = [make_shard(s) for s in self.slabs]

    def exchange(self) -> None:
        with _context(self.shards[0]):
            self._exchange()

    def _exchange(self) -> None:
        for s, sh in zip(self.slabs, self.shards):
            if s.right is not None:  # my last owned columns become the right neighbour's left halo
                self.shards[s.right].columns(0, s.rpad).copy_(sh.columns(s.lpad + s.own - s.rpad, s.rpad))
            if s.left is not None:  # my first owned columns become the left neighbour's right halo
                q = self.slabs[s.left]
                self.shards[s.left].columns(q.lpad + q.own, s.lpad).copy_(sh.columns(s.lpad, s.lpad))

    def run(self, t0: int, nsteps: int, params=None) -> None:
        t = int(t0)
        while nsteps > 0:
            k = min(self.K, nsteps)
            if len(self.slabs) > 1:
                self.exchange()
            for sh in self.shards:
                sh.step(t, k, params)
            t += k
            nsteps -= k

    def state(self) -> np.ndarray:
        n1, n2 = self.prob.space.dims
        out = np.empty((n1, n2), np.int8, order="F")
        for s, sh in zip(self.slabs, self.shards):
            out[:, s.j0:s.j1] = sh.read()[:, s.lpad:s.lpad + s.own]
        return out

    def summaries(self, nvals: int = 3):
        if len(self.slabs) > 1:
            self.exchange()
        total = sum(sh.sums(s.lpad, s.lpad + s.own) for s, sh in zip(self.slabs, self.shards))
        n1, n2 = self.prob.space.dims
        return summaries_from_sums(total, n1 * n2, nvals)

    def close(self):
        for sh in self.shards:
            close = getattr(sh, "close", None)
            if close:
                close()
