"""Stand-in for the parts of pandas the reference's src/class touches.

``DataFrame.to_csv`` writes nothing unless ``MCL_REFSHIM_CSV_DIR`` names a
directory: the reference writes into its own tree, which may be read-only,
so the file goes to that directory under the same base name.  The text
follows pandas 2.2.3 (the reference's pin, requirements.txt:14) for what the
reference writes (``to_csv(path, index=False)`` of integer and float64
columns): the column names joined by commas, then one line per row with
each integer column as ``str(int)`` and each float64 column as numpy's
``astype(str)`` (the shortest repr that round-trips), joined by commas,
every line ended by ``os.linesep``.  ``read_csv`` serves tables registered with ``register_table`` by the
fixture generator (synthetic lab tables), so the reference's TL_lab / ISO_lab
run unmodified on them.  The DataFrame supports what those methods use:
``iterrows`` with attribute access, column attributes with ``mean``,
``unique``, ``iloc`` and ``to_numpy``, and boolean row selection.
"""
import os

import numpy as np

_TABLES = {}


def register_table(name, columns):
    _TABLES[name] = {k: np.asarray(v) for k, v in columns.items()}


class Series(np.ndarray):
    def __new__(cls, a):
        return np.asarray(a).view(cls)

    @property
    def iloc(self):
        return _ILoc(self)

    def unique(self):
        out = []
        for v in np.asarray(self):
            if v not in out:
                out.append(v)
        return np.array(out)

    def to_numpy(self):
        return np.asarray(self).copy()

    def mean(self, *a, **k):
        return float(np.asarray(self).mean())


class _ILoc:
    def __init__(self, s):
        self.s = s

    def __getitem__(self, i):
        return np.asarray(self.s)[i].item()


class _Row:
    def __init__(self, d):
        self.__dict__.update(d)


class DataFrame(dict):
    def __init__(self, data=None, columns=None):
        super().__init__()
        if isinstance(data, dict):
            for k, v in data.items():
                self[k] = np.asarray(v)

    def __getattr__(self, k):
        try:
            return Series(self[k])
        except KeyError as e:
            raise AttributeError(k) from e

    def __getitem__(self, key):
        if isinstance(key, (np.ndarray, Series)) and np.asarray(key).dtype == bool:
            m = np.asarray(key)
            return DataFrame({k: np.asarray(v)[m] for k, v in self.items()})
        return dict.__getitem__(self, key)

    def iterrows(self):
        n = len(next(iter(self.values()))) if self else 0
        for i in range(n):
            yield i, _Row({k: np.asarray(v)[i].item() for k, v in self.items()})

    def to_csv(self, path=None, *a, index=True, **k):
        out_dir = os.environ.get("MCL_REFSHIM_CSV_DIR")
        if not out_dir or path is None:
            return None
        if index:
            raise NotImplementedError("the stand-in writes index=False tables only")
        cols = list(self.keys())
        text = [np.asarray(self[c]).astype(str) for c in cols]
        lines = [",".join(cols)] + [",".join(t[i] for t in text) for i in range(len(text[0]) if text else 0)]
        with open(os.path.join(out_dir, os.path.basename(str(path))), "w", newline="") as f:
            f.write(os.linesep.join(lines) + os.linesep)
        return None


def read_csv(path, *a, **k):
    name = os.path.splitext(os.path.basename(str(path)))[0]
    if name not in _TABLES:
        raise FileNotFoundError(path)
    return DataFrame(dict(_TABLES[name]))
