"""Model description for the sweep, mirroring the reference's types with the same names
and meaning: spaces and boundaries (src/spaces.jl), neighbourhoods
(src/neighbourhoods.jl), rules (src/rules.jl, src/lenia.jl), update schemes
(src/schemes.jl). Only what the GB300 sweep runs is here: two-dimensional square
lattices, Moore(r) / VonNeumann(r), Life / Generations / the forest-fire rule on Int8
states and Lenia on Float32 states."""
from __future__ import annotations

import math
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


class KernelSI:
    """The kernel-field SI epidemic of the reference's conformance battery
    (test/backend_conformance.jl:52-57 with a covariate, :72-75 in Float32) as a typed rule,
    on Int8 states:

        cell == 1 -> 1
        otherwise -> bernoulli(ctx, 1 - exp(-p.β * covariate(ctx, cov) * field(ctx, name))) ? 1 : cell

    `field` names a KernelField of the problem, `covariate` a covariate (None: the factor is
    left out). `float32=True` means β is Float32; products promote as in Julia (Float32 stays
    Float32 only against Float32)."""

    def __init__(self, field="pressure", covariate=None, float32: bool = False):
        self.field, self.covariate, self.float32 = field, covariate, float32
        self.neighbourhood = None

    def validate_state(self, u0):
        if not np.issubdtype(np.asarray(u0).dtype, np.integer):
            raise InvalidStateError("the kernel-field SI rule runs on integer (Int8) states")

    def __repr__(self):
        return f"KernelSI(field={self.field!r}, covariate={self.covariate!r})"


# ---------------------------------------------------------------- dispersal kernels (src/kernels.jl)


class GaussianKernel:
    """Weight exp(-d^2 / 2 sigma^2), cut off at radius = ceil(3 sigma) (kernels.jl:21-30)."""

    def __init__(self, sigma, radius=None):
        if not sigma > 0:
            raise ArgumentError(f"σ must be positive, got {sigma}")
        self.sigma = float(sigma)
        self.radius = int(math.ceil(3 * self.sigma)) if radius is None else int(radius)
        if self.radius < 1:
            raise ArgumentError(f"radius must be at least 1, got {self.radius}")

    def value(self, d, o):
        return math.exp(-(d * d) / (2 * (self.sigma * self.sigma)))


class ExponentialKernel:
    """Weight exp(-d / scale), cut off at radius = ceil(5 scale) (kernels.jl:38-47)."""

    def __init__(self, scale, radius=None):
        if not scale > 0:
            raise ArgumentError(f"scale must be positive, got {scale}")
        self.scale = float(scale)
        self.radius = int(math.ceil(5 * self.scale)) if radius is None else int(radius)
        if self.radius < 1:
            raise ArgumentError(f"radius must be at least 1, got {self.radius}")

    def value(self, d, o):
        return math.exp(-d / self.scale)


class PowerLawKernel:
    """Weight (1 + d)^(-alpha), cut off at radius = 10 (kernels.jl:55-64)."""

    def __init__(self, alpha, radius=10):
        if not alpha > 0:
            raise ArgumentError(f"α must be positive, got {alpha}")
        if radius < 1:
            raise ArgumentError(f"radius must be at least 1, got {radius}")
        self.alpha, self.radius = float(alpha), int(radius)

    def value(self, d, o):
        return math.pow(1.0 + d, -self.alpha)


class UniformKernel:
    """Equal weight within distance radius (kernels.jl:71-78)."""

    def __init__(self, radius):
        if radius < 1:
            raise ArgumentError(f"radius must be at least 1, got {radius}")
        self.radius = int(radius)

    def value(self, d, o):
        return 1.0


class LeniaKernel:
    """The smooth shell kernel of Lenia (kernels.jl:87-104)."""

    def __init__(self, R, peaks=(1.0,)):
        if R < 1:
            raise ArgumentError(f"R must be at least 1, got {R}")
        if len(peaks) < 1:
            raise ArgumentError("at least one peak is needed")
        self.radius, self.peaks = int(R), tuple(float(p) for p in peaks)

    def value(self, d, o):
        r = d / self.radius
        if r <= 0 or r >= 1:
            return 0.0
        B = len(self.peaks)
        x = B * r
        i = min(int(math.floor(x)), B - 1)
        f = x - i
        return self.peaks[i] * math.exp(4 - 1 / (f * (1 - f))) if 0 < f < 1 else 0.0


class AnisotropicKernel:
    """A base kernel tilted towards `direction` (radians; 0 = increasing column index, pi/2 =
    decreasing row index) by exp(strength cos(theta - direction)) (kernels.jl:115-132)."""

    def __init__(self, base, direction, strength):
        if not strength >= 0:
            raise ArgumentError(f"strength must be nonnegative, got {strength}")
        self.base, self.direction, self.strength = base, float(direction), float(strength)
        self.radius = base.radius

    def value(self, d, o):
        w = self.base.value(d, o)
        if d == 0:
            return w
        theta = math.atan2(-o[0], o[1])
        return w * math.exp(self.strength * math.cos(theta - self.direction))


class EmpiricalKernel:
    """A matrix of weights with odd sides, centred on the middle entry (kernels.jl:141-152)."""

    def __init__(self, weights):
        w = np.asarray(weights, dtype=np.float64)
        if w.ndim != 2 or not all(n % 2 == 1 for n in w.shape):
            raise ArgumentError(f"kernel matrix sides must be odd, got {w.shape}")
        if not (np.all(w >= 0) and np.all(np.isfinite(w))):
            raise ArgumentError("kernel weights must be finite and nonnegative")
        if not w.sum() > 0:
            raise ArgumentError("kernel weights must not all be zero")
        self.weights = w
        self.radius = max(n // 2 for n in w.shape)


def kernel_weights(kernel, space=None, include_centre: bool = True):
    """kernels.jl:174-203: the kernel's offsets (column-major order, first axis fastest) and
    their weights normalised to sum to one (a running sum, then one division each)."""
    offsets, weights = [], []
    if isinstance(kernel, EmpiricalKernel):
        c1, c2 = (kernel.weights.shape[0] + 1) // 2, (kernel.weights.shape[1] + 1) // 2
        for j in range(1, kernel.weights.shape[1] + 1):
            for i in range(1, kernel.weights.shape[0] + 1):
                o = (i - c1, j - c2)
                if o == (0, 0) and not include_centre:
                    continue
                w = float(kernel.weights[i - 1, j - 1])
                if w > 0:
                    offsets.append(o)
                    weights.append(w)
    else:
        r = kernel.radius
        for o2 in range(-r, r + 1):
            for o1 in range(-r, r + 1):
                if (o1, o2) == (0, 0) and not include_centre:
                    continue
                d = math.sqrt(float(o1 * o1) + float(o2 * o2))
                if not d <= r + 1e-9:
                    continue
                w = float(kernel.value(d, (o1, o2)))
                if w > 0:
                    offsets.append((o1, o2))
                    weights.append(w)
    if not weights:
        raise ArgumentError(f"kernel {kernel} has no positive weight")
    s = 0.0
    for w in weights:
        s += w
    return offsets, np.array([w / s for w in weights])


class KernelField:
    """KernelField(kernel, source; include_centre, method, precision) (environment.jl:22-41).
    `source` is "x == 1" (the indicator the conformance battery uses) or "identity"."""

    def __init__(self, kernel, source="identity", include_centre: bool = True, method: str = "direct",
                 precision: str = "Float64"):
        if method not in ("direct", "fft"):
            raise ArgumentError(f"method must be :direct or :fft, got :{method}")
        if source not in ("identity", "x == 1"):
            raise ArgumentError(f"GB300Backend reads fields with source identity or x == 1, got {source!r}")
        if precision not in ("Float32", "Float64"):
            raise ArgumentError(f"precision must be Float32 or Float64, got {precision}")
        self.kernel, self.source, self.include_centre = kernel, source, include_centre
        self.method, self.precision = method, precision

    def resolve(self, space, name):
        """environment.jl:53-69: (taps to read, weights, radius)."""
        offsets, weights = kernel_weights(self.kernel, space, include_centre=self.include_centre)
        taps = [(-a, -b) for a, b in offsets]
        if self.method == "fft" and not all(isinstance(b, Periodic) for b in space.boundaries):
            raise ArgumentError(f"field :{name} uses method=:fft, which needs periodic boundaries on every axis")
        radius = max(max(abs(a), abs(b)) for a, b in taps)
        return taps, weights, radius


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
