"""GB300-native Newton linear solver for ResSim Studio's black-oil engine (package placeholder; see solver.py)."""
from .bsr import BSR, NewtonSystem, ScalarCSR, load_npz, read_dump, read_system, save_npz  # noqa: F401
