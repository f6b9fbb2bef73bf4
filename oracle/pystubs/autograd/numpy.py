"""numpy re-export standing in for autograd.numpy (test infrastructure only)."""
from numpy import *  # noqa: F401,F403
from numpy import array, sin, cos, tan, arcsin, arccos, arctan, exp, log  # noqa: F401
