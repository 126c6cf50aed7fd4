"""evrgpu -- GB300 (sm_103a) H.psi path of ElVibRot-TnumTana behind a C ABI.

``Problem`` (evrgpu.lib) binds libevrgpu.so; ``evrgpu.spec`` describes bases and
operators and generates the seeded benchmark workloads.
"""
from .spec import ProblemSpec, AU_TO_CM, AU_TO_EV, FS_TO_AU  # noqa: F401
from .lib import Problem, BatchProblem, EvrError, load, library_path, EXPORTS  # noqa: F401
