"""Model description for the sweep, mirroring the reference's types with the same names
and meaning: spaces and boundaries (src/spaces.jl), neighbourhoods
(src/neighbourhoods.jl), rules (src/rules.jl, src/lenia.jl), update schemes
(src/schemes.jl). Only what the GB300 sweep runs is here: two-dimensional square
lattices, Moore(r) / VonNeumann(r), Life / Generations / the forest-fire rule on Int8
states and Lenia on Float32 states."""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

from .errors import ArgumentError, InvalidStateError, RuleParseError

# ---------------------------------------------------------------- boundaries and spaces


class Periodic:
    """The axis wraps around (src/spaces.jl:16)."""
    kind = 0

    def __repr__(self):
        return "Periodic()"


class Reflecting:
    """Mirrored at the edges, edge cell repeated (src/spaces.jl:25)."""
    kind = 1

    def __repr__(self):
        return "Reflecting()"


@dataclass(frozen=True)
class Constant:
    """Every cell beyond the edge holds `value` (src/spaces.jl:40-42)."""
    value: float = 0
    kind = 2


@dataclass(frozen=True)
class Lattice:
    """A two-dimensional square lattice with one boundary per axis (src/spaces.jl:94-110)."""
    dims: tuple
    boundaries: tuple

    def __post_init__(self):
        if len(self.dims) != 2:
            raise ArgumentError(f"GB300Backend runs two-dimensional lattices, got {len(self.dims)} dimensions")
        if not all(d > 0 for d in self.dims):
            raise ArgumentError(f"lattice dimensions must be positive, got {self.dims}")
        if len(self.boundaries) != 2:
            raise ArgumentError("need one boundary per axis (2)")

    def size(self):
        return self.dims


def _bnds(b):
    return tuple(b) if isinstance(b, (tuple, list)) else (b, b)


def Torus(*dims) -> Lattice:
    """Periodic on every axis (src/spaces.jl:130-131)."""
    dims = tuple(dims[0]) if len(dims) == 1 and isinstance(dims[0], tuple) else tuple(int(d) for d in dims)
    return Lattice(dims, (Periodic(), Periodic()))


def Grid(*dims, boundary=Constant(0)) -> Lattice:
    """A lattice with edges, Constant(0) by default (src/spaces.jl:140-143)."""
    dims = tuple(dims[0]) if len(dims) == 1 and isinstance(dims[0], tuple) else tuple(int(d) for d in dims)
    return Lattice(dims, _bnds(boundary))


# ---------------------------------------------------------------- neighbourhoods


@dataclass(frozen=True)
class Moore:
    """Chebyshev distance <= radius (src/neighbourhoods.jl:21-27)."""
    radius: int = 1

    def __post_init__(self):
        if self.radius < 1:
            raise ArgumentError(f"Moore radius must be at least 1, got {self.radius}")

    kind = 1


@dataclass(frozen=True)
class VonNeumann:
    """Manhattan distance <= radius (src/neighbourhoods.jl:35-42)."""
    radius: int = 1

    def __post_init__(self):
        if self.radius < 1:
            raise ArgumentError(f"von Neumann radius must be at least 1, got {self.radius}")

    kind = 2


def neighbourhood_offsets(n, space=None):
    """Column-major offsets, centre excluded (src/neighbourhoods.jl:124-153)."""
    r = n.radius
    out = []
    for dj in range(-r, r + 1):
        for di in range(-r, r + 1):
            if (di, dj) == (0, 0):
                continue
            if isinstance(n, VonNeumann) and abs(di) + abs(dj) > r:
                continue
            out.append((di, dj))
    return out


# ---------------------------------------------------------------- rules

LIFE_PRESETS = {"conway": "B3/S23", "highlife": "B36/S23", "seeds": "B2/S", "day_and_night": "B3678/S34678",
                "morley": "B368/S245", "two_by_two": "B36/S125", "replicator": "B1357/S1357",
                "diamoeba": "B35678/S5678", "thirty_four": "B34/S34", "life_without_death": "B3/S012345678",
                "maze": "B3/S12345"}
GENERATIONS_PRESETS = {"brians_brain": "B2/S/C3", "star_wars": "B2/S345/C4"}


def _mask(counts, rule) -> int:
    m = 0
    for c in counts:
        if not 0 <= c <= 63:
            raise ArgumentError(f"neighbour counts must be in 0:63, got {c} in {rule}")
        m |= 1 << int(c)
    return m


def _counts(m: int):
    return [c for c in range(64) if (m >> c) & 1]


def _digitstring(m: int) -> str:
    cs = _counts(m)
    if all(c <= 8 for c in cs):
        return "".join(str(c) for c in cs)
    runs, i = [], 0
    while i < len(cs):
        j = i
        while j < len(cs) - 1 and cs[j + 1] == cs[j] + 1:
            j += 1
        runs.append(f"{cs[i]}..{cs[j]}" if j > i else str(cs[i]))
        i = j + 1
    return ",".join(runs)


def _parse_digits(s, rule):
    for ch in s:
        if not "0" <= ch <= "8":
            raise RuleParseError(f"{rule}: neighbour counts in a rule string are digits 0 to 8, got '{ch}'")
    return [int(ch) for ch in s]


def _parse_rule(text: str):
    """src/rules.jl:316-330: B/S or S/B notation, with an optional /C."""
    s = re.sub(r"\s", "", text).upper()
    m = re.fullmatch(r"B([0-9]*)/?S([0-9]*)(?:/C?([0-9]+))?", s)
    if m:
        c = None if m.group(3) is None else int(m.group(3))
        return _parse_digits(m.group(1), text), _parse_digits(m.group(2), text), c
    m = re.fullmatch(r"([0-9]*)/([0-9]*)(?:/([0-9]+))?", s)
    if m:
        c = None if m.group(3) is None else int(m.group(3))
        return _parse_digits(m.group(2), text), _parse_digits(m.group(1), text), c
    raise RuleParseError(f"{text}: expected B/S notation such as \"B3/S23\" or S/B notation such as \"23/3\"")


def _preset(rule, presets, what):
    """A preset name ("highlife", or ":highlife" for Julia's Symbol :highlife) becomes its
    rule string; an unknown ":name" is an ArgumentError, as for an unknown Symbol."""
    name = str(rule)
    if name.startswith(":"):
        if name[1:] not in presets:
            raise ArgumentError(f"unknown {what} preset {name}; known presets are {sorted(presets)}")
        return presets[name[1:]]
    return presets.get(name, name)


class Life:
    """Two-state outer-totalistic rule (src/rules.jl:354-389): Life("B36/S23"),
    Life("highlife"), or Life(birth_counts, survive_counts; neighbourhood)."""

    def __init__(self, rule="B3/S23", survive=None, neighbourhood=None):
        if survive is not None:
            self.birth, self.survive = _mask(rule, "Life"), _mask(survive, "Life")
        else:
            rule = _preset(rule, LIFE_PRESETS, "Life")
            b, s, c = _parse_rule(rule)
            if c is not None and c != 2:
                raise RuleParseError(f"{rule}: a Life rule has two states; use Generations for C{c}")
            self.birth, self.survive = _mask(b, rule), _mask(s, rule)
        self.neighbourhood = neighbourhood

    def validate_state(self, u0):
        """src/rules.jl:391: states 0 and 1."""
        _check_values(self, u0, (0, 1), "a Life rule has states 0 and 1")

    def rulestring(self):
        return "B" + _digitstring(self.birth) + "/S" + _digitstring(self.survive)

    def __repr__(self):
        return f"Life({self.rulestring()!r})"


class Generations:
    """Generations rule with C states (src/rules.jl:424-456)."""

    def __init__(self, rule, neighbourhood=None):
        rule = _preset(rule, GENERATIONS_PRESETS, "Generations")
        b, s, c = _parse_rule(rule)
        if c is None:
            raise RuleParseError(f"{rule}: a Generations rule needs a state count, as in \"B2/S/C3\"")
        if c < 2:
            raise RuleParseError(f"{rule}: a Generations rule needs at least 2 states")
        self.birth, self.survive, self.states = _mask(b, rule), _mask(s, rule), c
        self.neighbourhood = neighbourhood

    def validate_state(self, u0):
        _check_values(self, u0, range(self.states), f"states must be in 0:{self.states - 1}")

    def rulestring(self):
        return "B" + _digitstring(self.birth) + "/S" + _digitstring(self.survive) + "/C" + str(self.states)

    def __repr__(self):
        return f"Generations({self.rulestring()!r})"


class ForestFire:
    """The forest-fire LocalRule of the package README on Int8 codes 0 (empty), 1 (tree),
    2 (fire), with p = (p=..., f=...):

        cell == 2 -> 0
        cell == 0 -> bernoulli(ctx, p.p, 1) ? 1 : 0
        otherwise -> any neighbour == 2 ? 2 : (bernoulli(ctx, p.f, 2) ? 2 : 1)

    A typed rule, so that its Julia counterpart's `local_rule` is the same code the
    ReferenceBackend runs. `float32=True` means p and f are Float32 (random.jl:130)."""

    def __init__(self, neighbourhood=None, float32: bool = False):
        self.neighbourhood = neighbourhood if neighbourhood is not None else VonNeumann(1)
        self.float32 = float32

    def validate_state(self, u0):
        pass

    def __repr__(self):
        return f"ForestFire({self.neighbourhood})"


class Lenia:
    """Lenia (src/lenia.jl:17-47): potential U from the LeniaKernel(R; peaks) field, then
    clamp(c + dt (2 exp(-(U - mu)^2 / 2 sigma^2) - 1), 0, 1), in the precision of the
    state (precision="Float32" or "Float64", as the reference's `precision` keyword)."""

    def __init__(self, R=13, mu=0.15, sigma=0.015, dt=0.1, peaks=(1.0,), method="direct", precision="Float64"):
        if not sigma > 0:
            raise ArgumentError(f"σ must be positive, got {sigma}")
        if not 0 < dt <= 1:
            raise ArgumentError(f"dt must be in (0, 1], got {dt}")
        if method not in ("direct", "fft"):
            raise ArgumentError(f"method must be :direct or :fft, got :{method}")
        if precision not in ("Float32", "Float64"):
            raise ArgumentError(f"precision must be Float32 or Float64, got {precision}")
        if R < 1:
            raise ArgumentError(f"R must be at least 1, got {R}")
        if len(peaks) < 1:
            raise ArgumentError("at least one peak is needed")
        self.R, self.mu, self.sigma, self.dt = int(R), float(mu), float(sigma), float(dt)
        self.peaks, self.method, self.neighbourhood = tuple(float(x) for x in peaks), method, None
        self.precision = precision

    def validate_state(self, u0):
        if not np.issubdtype(np.asarray(u0).dtype, np.floating):
            raise InvalidStateError("Lenia needs a floating-point state")
        a = np.asarray(u0)
        if not np.all((a >= 0) & (a <= 1)):
            raise InvalidStateError("states must be in [0, 1]")

    def __repr__(self):
        return f"Lenia(R={self.R}, μ={self.mu}, σ={self.sigma}, dt={self.dt})"


def _check_values(rule, u0, allowed, msg):
    a = np.asarray(u0)
    bad = ~np.isin(a, np.asarray(list(allowed)))
    if bad.any():
        idx = tuple(int(x) + 1 for x in np.argwhere(bad)[0])
        raise InvalidStateError(f"{rule}: cell {idx} holds {a[tuple(i - 1 for i in idx)]}: {msg}")


# ---------------------------------------------------------------- schemes


class Synchronous:
    """All cells update at once (src/schemes.jl:22)."""

    def __repr__(self):
        return "Synchronous()"


class Stochastic:
    """Each cell updates with probability p, decided by its draw k = 0 (src/schemes.jl:33-40)."""

    def __init__(self, p, float32: bool = False):
        if not 0 < p <= 1:
            raise ArgumentError(f"update probability must be in (0, 1], got {p}")
        self.p, self.float32 = float(np.float32(p)) if float32 else float(p), float32

    def __repr__(self):
        return f"Stochastic({self.p})"


class Checkerboard:
    """Even index sums first, then odd ones, each half reading the other's result
    (src/schemes.jl:51)."""

    def __repr__(self):
        return "Checkerboard()"
