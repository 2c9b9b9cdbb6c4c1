"""Import stand-in for ``PyWavelets`` (test infrastructure only).

On the default BM3D/BM4D path the reference consults PyWavelets only for
``Wavelet(name).orthogonal`` because the bior1.5 matrices for lengths 4 and 8
are tabulated in its own source.  Anything that needs real filter banks raises.
"""


class Wavelet:
    def __init__(self, name):
        self.name = name
        self.orthogonal = name in ("haar", "db1")
        self.dec_lo = [0.0, 0.0]


def dwt_max_level(data_len, filter_len):
    raise NotImplementedError("filter banks are not available in the oracle shim")


def wavedec(*args, **kwargs):
    raise NotImplementedError("filter banks are not available in the oracle shim")
