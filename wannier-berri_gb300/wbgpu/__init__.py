"""wbgpu: GB300-native (sm_103a) Wannier-interpolation backend.

Host-side mirror of the reference interface for the hot path -- ``System_R``,
``Grid``, ``run`` and the calculators -- over hand-written CUDA kernels reached
through the C ABI of libwbgpu.so (include/wbgpu.h).
"""
from .system import System_R
from .grid import Grid
from .run import run, run_refine_omega
from . import calculators, models, engine, serve, autotune, distributed
from .result import EnergyResult, ResultDict
from .serve import Server, run_many
from .tabulate import evaluate_k, tabulate

__all__ = ['System_R', 'Grid', 'run', 'run_refine_omega', 'calculators', 'models', 'engine', 'serve', 'autotune', 'distributed', 'Server',
           'run_many', 'evaluate_k', 'tabulate', 'EnergyResult', 'ResultDict']
