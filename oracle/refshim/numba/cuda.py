"""numba.cuda stand-in: the reference's CUDA branch is never taken here
(``env.platform`` stays 'CPU'); these names only need to exist."""


def jit(*args, **kwargs):
    def deco(func):
        return func

    return deco


def to_device(array):
    raise RuntimeError("numba.cuda is not available in this environment")


class atomic:  # noqa: N801
    @staticmethod
    def add(*args, **kwargs):
        raise RuntimeError("numba.cuda is not available in this environment")


blockIdx = blockDim = threadIdx = None
