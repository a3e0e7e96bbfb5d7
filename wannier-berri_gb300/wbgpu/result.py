"""Result container mirroring the reference ``EnergyResult`` (result/energyresult.py:11-278):
data tabulated against one or more energy axes (Fermi levels [, frequencies])."""
import numpy as np


class EnergyResult:
    def __init__(self, Energies, data, comment=""):
        self.Energies = list(Energies) if isinstance(Energies, (list, tuple)) else [Energies]
        self.data = np.asarray(data)
        self.comment = comment

    @property
    def N_energies(self):
        return len(self.Energies)

    def __add__(self, other):
        if other is None or (isinstance(other, (int, float)) and other == 0):
            return self
        for a, b in zip(self.Energies, other.Energies):
            if np.linalg.norm(np.asarray(a) - np.asarray(b)) > 1e-8:
                raise RuntimeError("Adding results with different energies - not allowed")
        return EnergyResult(self.Energies, self.data + other.data, self.comment)

    def __radd__(self, other):
        return self.__add__(other)

    def __mul__(self, number):
        if isinstance(number, (int, float, np.floating, np.integer)):
            return EnergyResult(self.Energies, self.data * number, self.comment)
        raise TypeError("result can only be multiplied by a number")

    __rmul__ = __mul__

    def __sub__(self, other):
        return self + (-1) * other

    def mul_array(self, other, axes=None):
        other = np.asarray(other)
        if isinstance(axes, int):
            axes = (axes,)
        if axes is None:
            axes = tuple(range(other.ndim))
        reshape = tuple((self.data.shape[i] if i in axes else 1) for i in range(self.data.ndim))
        return EnergyResult(self.Energies, self.data * other.reshape(reshape), self.comment)

    def add(self, other):
        self.data = self.data + other.data

    @property
    def max(self):
        """EnergyResult.max (result/energyresult.py:250-264, no smoothers): max |data|, its 2-norm
        and the 2-norm of its difference along the first energy axis -- the numbers by which
        adaptive refinement ranks K-points."""
        d = self.data
        return np.array([np.abs(d).max(), np.linalg.norm(d), np.linalg.norm(d[1:] - d[:-1])])

    def savedata(self, name, prefix="", suffix="", i_iter=0):
        """Binary output like EnergyResult.save (npz with data and energy axes)."""
        fn = f"{prefix}-{name}{('-' + suffix) if suffix else ''}_iter-{i_iter:04d}.npz"
        np.savez_compressed(fn, data=self.data, **{f"Energies_{i}": E for i, E in enumerate(self.Energies)})
        return fn


class ResultDict(dict):
    """Mapping calculator key -> EnergyResult (result/resultdict.py:18-66)."""

    @property
    def results(self):
        return self

    @property
    def max(self):
        """ResultDict.max (result/resultdict.py:62-63): the max entries of every result in order."""
        return np.array([x for v in self.values() for x in v.max])
