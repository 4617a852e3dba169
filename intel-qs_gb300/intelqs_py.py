"""`import intelqs_py as iqs` for programs written against intel-qs's Python module
(pybind11/intelqs_py.cpp): the same names, backed by iqs_gb300 and the GPU."""
from iqs_gb300 import *  # noqa: F401,F403
from iqs_gb300 import __all__  # noqa: F401
