"""adpy.variable names, served by the stand-in in adpy.tensor."""
from .tensor import Variable, StaticVariable, StaticIntegerVariable, IntegerScalar, Zeros, Function, Kernel, Container  # noqa: F401
