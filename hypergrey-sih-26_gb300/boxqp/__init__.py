"""GB300 box-constrained convex QP engine (host layer over libboxqp.so)."""
from ._native import EngineError, LIB_PATH, Options, PlantedSpec, Stats, STATUS_NAMES, lib
from .api import (BoxIteration, Engine, QpOptions, QpResult, QuadraticProblem, check_convex_hessian,
                  csr_from_lower, cuda_device_name, default_engine, gershgorin, make_cuda_box, options_struct,
                  pinned, planted, planted_spec, problem_from_planted, solve_accelerated_box, splitmix64)

__all__ = ['BoxIteration', 'Engine', 'EngineError', 'LIB_PATH', 'Options', 'PlantedSpec', 'QpOptions', 'QpResult',
           'QuadraticProblem', 'STATUS_NAMES', 'Stats', 'check_convex_hessian', 'csr_from_lower',
           'cuda_device_name', 'default_engine', 'gershgorin', 'lib', 'make_cuda_box', 'options_struct', 'pinned', 'planted',
           'planted_spec', 'problem_from_planted', 'solve_accelerated_box', 'splitmix64']
