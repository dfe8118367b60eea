"""Exception types of the reference's error tree (src/errors.jl) that this backend raises,
plus the device-side failures the C ABI reports."""


class CellularAutomataCoreError(Exception):
    """Supertype of the package's own errors (src/errors.jl)."""


class ArgumentError(ValueError):
    """Julia's ArgumentError."""


class IncompatibleSpaceError(CellularAutomataCoreError):
    """A neighbourhood, boundary or scheme does not fit the space."""


class UnsupportedCombinationError(CellularAutomataCoreError):
    """The backend cannot run the scheme (src/errors.jl:124-132)."""

    def __init__(self, backend, scheme=None):
        super().__init__(backend if scheme is None else f"{backend} cannot run {scheme}")


class StateShapeError(CellularAutomataCoreError):
    """A state, mask or covariate has the wrong size."""


class InvalidStateError(CellularAutomataCoreError):
    """The rule cannot read a value of the initial state."""


class RuleParseError(CellularAutomataCoreError):
    """A rule string is not in B/S or S/B notation."""


class GPUError(RuntimeError):
    """A CUDA failure, or the library is missing."""


class OutOfDeviceMemory(GPUError):
    """Device memory or an admission budget is exhausted."""


class DeviceTimeout(GPUError):
    """A bounded device-side wait gave up."""


class Busy(GPUError):
    """A queue is full; retry later."""
