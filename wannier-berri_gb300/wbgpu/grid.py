"""K-point grid mirror (grid/grid.py:86-189, grid/Kpoint.py:104-175): NKdiv x NKFFT blocks.

Each K-point of the division grid is one FFT block whose k-points are
j/NKFFT + K/NKFFT (j in C order); its weight in run() is 1/prod(NKdiv).
"""
import numpy as np


def _three(x):
    if x is None:
        return None
    a = np.array([x] * 3 if np.ndim(x) == 0 else x, dtype=int)
    assert a.shape == (3,) and np.all(a > 0)
    return a


class Grid:
    def __init__(self, system=None, NKdiv=None, NKFFT=None, NK=None, length=None, use_symmetry=False, **_):
        NKdiv, NKFFT, NK = _three(NKdiv), _three(NKFFT), _three(NK)
        if NKFFT is None:
            NKFFT = np.array(system.NKFFT_recommended) if system is not None else None
        if NKdiv is None:
            if NK is None or NKFFT is None:
                raise ValueError("you need to specify either NK or a pair (NKdiv,NKFFT) or (NK,NKFFT)")
            NKdiv = np.maximum(np.round(NK / NKFFT).astype(int), 1)
        self.div = NKdiv
        self.FFT = NKFFT
        if system is not None:
            notper = ~np.asarray(system.periodic, dtype=bool)
            self.div[notper] = 1
            self.FFT[notper] = 1

    @property
    def dense(self):
        return self.div * self.FFT

    @property
    def nk_per_block(self):
        return int(np.prod(self.FFT))

    @property
    def nblocks(self):
        return int(np.prod(self.div))

    def block_shifts(self):
        """dK = K/NKFFT for every K of the division grid (Kpoint.Kp_fullBZ), C order."""
        g = np.stack(np.meshgrid(*[np.arange(n) for n in self.div], indexing='ij'), axis=-1).reshape(-1, 3)
        return (g / self.div[None, :]) / self.FFT[None, :]

    @property
    def str_short(self):
        return f"Grid() with NKdiv={self.div}, NKFFT={self.FFT}, NKtot={self.dense}"
