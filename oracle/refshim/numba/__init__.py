"""Minimal stand-in for numba, used only to run the unmodified reference
package (mdpy v0.2.1) on the CPU in a container that has no numba.

It makes ``nb.njit(...)`` an identity decorator -- exactly the mode the
reference's own test runner selects with ``NUMBA_DISABLE_JIT=1``
(mdpy/test/run_test.py:63) -- and gives the dtype names that appear in the
reference's jit signatures something subscriptable to stand on.
Test infrastructure only: nothing in the shipped package imports this.
"""


class _Type:
    def __init__(self, name):
        self.name = name

    def __getitem__(self, _):
        return self

    def __call__(self, *args, **kwargs):
        return self

    def __repr__(self):
        return "<numba-stub type %s>" % self.name


float32 = _Type("float32")
float64 = _Type("float64")
int32 = _Type("int32")
int64 = _Type("int64")
void = _Type("void")


def njit(*args, **kwargs):
    # @njit  /  @njit()  /  njit(signature)(func)
    if len(args) == 1 and callable(args[0]) and not isinstance(args[0], _Type) and not kwargs:
        return args[0]

    def deco(func):
        return func

    return deco


jit = njit

from . import cuda  # noqa: E402,F401
