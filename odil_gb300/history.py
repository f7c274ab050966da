"""Per-epoch history table with CSV output (util_history.py:7-108).

Columns are appended value by value; ``commit`` closes a row; ``write``
commits and appends the rows not yet written to the CSV file (the header is
the column order of the first written row).  A column that first appears
after some rows is back-filled with zeros of the value's kind, as the
reference does, and a row that misses a column is an error.  ``save``/``load``
store the columns as a pickled dict of lists, the reference's file layout.
"""
import pickle

import numpy as np

_SCALARS = (int, float, str, np.float32, np.float64)


def _zero_of(value):
    if value is None:
        return None
    if isinstance(value, (bool, np.bool_)):
        raise TypeError("unexpected type: %s" % type(value))
    if isinstance(value, int):
        return 0
    if isinstance(value, (float, np.floating)):
        return 0.
    return None  # strings: the reference back-fills nothing meaningful


class History:

    def __init__(self, csvpath=None, warmup=0):
        """warmup: rows are written only once more than `warmup` exist."""
        self.data = {}
        self.count = 0
        self.warmup = warmup
        self.csvpath = csvpath
        self.csvkeys = None
        self.csvcount = 0
        self.csvfile = open(csvpath, "w") if csvpath is not None else None

    def append(self, key, value=None):
        if value is not None and type(value) not in _SCALARS:
            raise TypeError("unexpected type: %s" % type(value))
        col = self.data.get(key)
        if col is None:
            if value is None:
                raise ValueError("first value of column %r is None" % key)
            col = self.data[key] = [_zero_of(value)] * self.count
        if value is None:
            if not col:
                raise ValueError("expected non-empty column " + key)
            value = _zero_of(col[-1])
        col.append(value)

    def append_dict(self, values):
        for key, value in values.items():
            self.append(key, value)

    def get(self, key, default=None):
        return self.data.get(key, default)

    def commit(self):
        """Closes the current row; every column must have a value in it."""
        n = max((len(c) for c in self.data.values()), default=0)
        short = [k for k, c in self.data.items() if len(c) < n]
        if short:
            raise RuntimeError("Missing values for columns: " +
                               ",".join(short) + ",")
        self.count += 1

    def write(self, nocommit=False):
        """Commits (unless `nocommit`) and writes the pending rows."""
        if not nocommit:
            self.commit()
        if self.count <= self.warmup or self.csvfile is None:
            return
        if self.csvkeys is not None and len(self.csvkeys) != len(self.data):
            extra = sorted(set(self.data) - set(self.csvkeys))
            raise RuntimeError("Unexpected keys in history: %s" % extra)
        if self.csvcount == 0:
            self.csvkeys = list(self.data)
            self.csvfile.write(",".join(self.csvkeys) + "\n")
        lines = []
        for r in range(self.csvcount, self.count):
            lines.append(",".join(str(self.data[k][r]) for k in self.data))
        if lines:
            self.csvfile.write("\n".join(lines) + "\n")
        self.csvcount = self.count
        self.csvfile.flush()

    def save(self, path):
        with open(path, "wb") as f:
            pickle.dump(self.data, f)

    def load(self, path):
        """Replaces the columns with a saved table and writes its rows."""
        with open(path, "rb") as f:
            self.data = pickle.load(f)
        self.csvkeys = list(self.data)
        self.count = len(next(iter(self.data.values()))) if self.data else 0
        self.write(nocommit=True)

    def close(self):
        if self.csvfile is not None:
            self.csvfile.close()
            self.csvfile = None
