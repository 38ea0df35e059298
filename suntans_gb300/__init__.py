"""GB300-native elliptic solvers for SUNTANS (CGSolveQ / CGSolve drop-in)."""
from .grid import SunGrid, QProblem, HProblem, SolverProps  # noqa: F401
