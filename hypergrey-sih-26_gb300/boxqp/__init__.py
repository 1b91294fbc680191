"""GB300 box-constrained convex QP engine (host layer over libboxqp.so)."""
from ._native import EngineError, LIB_PATH, Options, PlantedSpec, Stats, STATUS_NAMES, lib
from .api import (BoxIteration, Engine, QpOptions, QpResult, QuadraticProblem, check_convex_hessian,
                  csr_from_lower, cuda_device_name, default_engine, gershgorin, make_cuda_box, options_struct,
                  pinned, planted, planted_spec, problem_from_planted, solve_accelerated_box, splitmix64)
from .admm import AdmmSystem, LinearRows, solve_qp_admm

__all__ = ['AdmmSystem', 'BoxIteration', 'Engine', 'EngineError', 'LIB_PATH', 'Options', 'PlantedSpec', 'QpOptions', 'QpResult',
           'QuadraticProblem', 'LinearRows', 'STATUS_NAMES', 'Stats', 'check_convex_hessian', 'csr_from_lower',
           'cuda_device_name', 'default_engine', 'gershgorin', 'lib', 'make_cuda_box', 'options_struct', 'pinned', 'planted',
           'planted_spec', 'problem_from_planted', 'solve_accelerated_box', 'solve_qp_admm', 'splitmix64']
