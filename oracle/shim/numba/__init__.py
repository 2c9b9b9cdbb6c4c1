"""Import stand-in for ``numba`` so the reference package runs as plain Python.

Test infrastructure only: the golden-vector generator puts this directory first
on ``sys.path`` together with the reference's ``src`` tree.  ``njit`` returns
the function unchanged, ``prange`` is ``range`` and the thread-count helpers
report one thread, so every ``@njit`` loop of the reference executes with
NumPy scalar semantics (float32 arithmetic stays float32).
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(func):
        return func

    return wrap


jit = njit
prange = range


def get_num_threads():
    return 1


def set_num_threads(n):
    return None
