"""GB300 backend for CellularAutomataCore.jl's synchronous halo-padded stencil sweep.

The compute path is libgbca.so (hand-written sm_103a CUDA, C ABI in include/gbca.h);
this package is the host-side mirror of the reference's interface over it:
model types (spaces, neighbourhoods, rules, schemes), the backend contract
(GB300Backend and its functions) and the SciML-style problem / solve layer."""
from . import backend, capi, ensemble, errors, model, problem, serving, slabs
from .backend import (GB300Backend, GB300State, advance, allocate_state, check_problem, current_state,
                      device_summaries, read_cell, set_geometry, set_state, supports, tune, update_cell,
                      write_cell)
from .errors import (ArgumentError, GPUError, IncompatibleSpaceError, InvalidStateError, RuleParseError,
                     StateShapeError, UnsupportedCombinationError)
from .model import (GENERATIONS_PRESETS, LIFE_PRESETS, AnisotropicKernel, Checkerboard, Constant, EmpiricalKernel,
                    ExponentialKernel, ForestFire, GaussianKernel, Generations, Grid, KernelField, KernelSI, Lattice,
                    Lenia, LeniaKernel, Life, Moore, Periodic, PowerLawKernel, Reflecting, Stochastic, Synchronous,
                    Torus, UniformKernel, VonNeumann, kernel_weights, neighbourhood_offsets)
from .problem import (CAProblem, CASolution, DiscreteCallback, EnsembleProblem, final_state, init, reinit, remake,
                      seed_trajectory, solve, solve_ensemble_serial, solve_integrator, step)

from .serving import Server
from .ensemble import ABCResult, BatchedEnsemble, EnsembleGB300, EnsembleResult, abc_rejection, solve_ensemble

__version__ = "0.1.0"
