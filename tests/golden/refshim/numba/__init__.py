"""No-op stand-in for numba: the reference's numba backend module is imported
unconditionally (shenfun/optimization/__init__.py:18) but only used when
config['optimization']['mode'] == 'numba'; the golden runs use 'cython'."""


def _decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(f):
        return f
    return wrap


jit = njit = vectorize = guvectorize = generated_jit = _decorator
prange = range


class _Any:
    def __getattr__(self, name):
        return _Any()

    def __call__(self, *a, **k):
        return _Any()

    def __getitem__(self, k):
        return _Any()


types = _Any()
int64 = int32 = float64 = float32 = complex128 = boolean = void = _Any()


class _Errors:
    class NumbaPerformanceWarning(Warning):
        pass


class core:  # noqa: N801
    errors = _Errors
