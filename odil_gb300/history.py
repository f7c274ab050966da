"""Training history: a table of per-epoch scalars, written as CSV.

The file formats follow the reference's history (util_history.py:7-108),
since drivers and plotting scripts read them:

* the table is a dict that maps a column name to the list of its values, one
  value per committed row, in the order the columns first appeared; the
  pickle file (``save`` / ``load``) is exactly that dict;
* the CSV file has a header line of the column names, fixed by the first
  write, then one line per row with each value formatted by ``str``, values
  separated by commas and no quoting; rows are appended as they are
  committed, once more than ``warmup`` rows exist;
* a column that first appears after k rows holds k zeros of its first
  value's kind before that value (0 for integers, 0.0 for floats, None for
  strings), and a value of None stands for the zero of the column's kind.

Everything else here (the pending-row check, the CSV writer) is this
engine's own.
"""
import pickle

import numpy as np


def _kind_zero(value):
    """The zero that stands in for a missing value of `value`'s kind."""
    if isinstance(value, (bool, np.bool_)):
        raise TypeError("history values are numbers or strings, not %s"
                        % type(value).__name__)
    if isinstance(value, (int, np.integer)):
        return 0
    if isinstance(value, (float, np.floating)):
        return 0.0
    return None


def _accepts(value):
    return value is None or isinstance(
        value, (int, float, str, np.integer, np.floating)) and not isinstance(
            value, (bool, np.bool_))


class _CsvSink:
    """Appends committed rows to a CSV file; the header is the column list
    at the first write and cannot grow afterwards."""

    def __init__(self, path):
        self.stream = open(path, "w")
        self.header = None
        self.rows_out = 0

    def emit(self, table, nrows):
        names = list(table)
        if self.header is None:
            self.header = names
            self.stream.write(",".join(names) + "\n")
        elif names != self.header:
            added = [k for k in names if k not in self.header]
            raise RuntimeError("columns %s appeared after the CSV header "
                               "was written" % ", ".join(map(repr, added)))
        out = []
        for r in range(self.rows_out, nrows):
            out.append(",".join(str(table[k][r]) for k in names) + "\n")
        self.stream.write("".join(out))
        self.stream.flush()
        self.rows_out = nrows

    def close(self):
        self.stream.close()


class History:
    """Per-epoch scalars: ``append`` values to the open row, ``commit`` the
    row, ``write`` commits and appends the new rows to the CSV file."""

    def __init__(self, csvpath=None, warmup=0):
        self.data = {}
        self.count = 0
        self.warmup = warmup
        self._csv = _CsvSink(csvpath) if csvpath is not None else None

    def append(self, key, value=None):
        """Puts `value` in column `key` of the open row."""
        if not _accepts(value):
            raise TypeError("history values are numbers or strings, not %s"
                            % type(value).__name__)
        values = self.data.get(key)
        if values is None:
            if value is None:
                raise ValueError("column %r has no value to take its kind "
                                 "from" % key)
            zero = _kind_zero(value)
            self.data[key] = values = [zero for _ in range(self.count)]
        elif value is None:
            if not values:
                raise ValueError("column %r has no value to take its kind "
                                 "from" % key)
            value = _kind_zero(values[-1])
        values.append(value)

    def append_dict(self, values):
        for key, value in values.items():
            self.append(key, value)

    def get(self, key, default=None):
        return self.data.get(key, default)

    def commit(self):
        """Closes the open row; each column must have received a value."""
        lacking = [k for k, v in self.data.items() if len(v) <= self.count]
        if lacking and len(lacking) < len(self.data):
            raise RuntimeError("row %d has no value for %s"
                               % (self.count, ", ".join(map(repr, lacking))))
        self.count += 1

    def write(self, nocommit=False):
        """Commits the open row (unless `nocommit`) and appends the rows not
        yet in the CSV file, once more than `warmup` rows exist."""
        if not nocommit:
            self.commit()
        if self._csv is not None and self.count > self.warmup:
            self._csv.emit(self.data, self.count)

    def save(self, path):
        with open(path, "wb") as f:
            pickle.dump(self.data, f)

    def load(self, path):
        """Replaces the table with a saved one and writes its rows."""
        with open(path, "rb") as f:
            table = pickle.load(f)
        lengths = {len(v) for v in table.values()}
        if len(lengths) > 1:
            raise ValueError("columns of %s differ in length: %s"
                             % (path, sorted(lengths)))
        self.data = table
        self.count = lengths.pop() if lengths else 0
        self.write(nocommit=True)

    def close(self):
        if self._csv is not None:
            self._csv.close()
            self._csv = None
