"""qsl's benchmark Results table (include/qsl/benchmark/results.hpp:49-246,
results.tpp), for writing GPU timings in the file format qsl's own
benchmarks write and its plotting script reads (comment lines starting
with '#', then whitespace-separated columns).

The integer columns come first in every row, then the floating-point ones,
as in the reference; numbers are printed as a C++ std::ostream prints
them by default (integers in decimal, floating point as %g with 6
significant digits)."""
from __future__ import annotations

import math


class Results:
    """Results<T, R>: a table of integer and floating-point columns plus
    metadata lines (results.tpp:30-355)."""

    def __init__(self, headings):
        self.head = list(headings)
        self.meta: list[str] = []
        self.intcols: list[list[int]] = []
        self.fpcols: list[list[float]] = []

    # results.tpp:72-103
    def addRow(self, ints, fps) -> None:
        ints, fps = [int(x) for x in ints], [float(x) for x in fps]
        if not self.intcols:
            if len(ints) + len(fps) != len(self.head):
                raise ValueError("Total number of columns does not match number of column "
                                 "headings in first call to addRow")
        else:
            if len(self.intcols[0]) != len(ints):
                raise ValueError("Incorrect number of integer columns in call to addRow")
            if len(self.fpcols[0]) != len(fps):
                raise ValueError("Incorrect number of floating point columns in call to addRow")
        self.intcols.append(ints)
        self.fpcols.append(fps)

    def addMeta(self, line: str) -> None:
        self.meta.append(str(line))

    def getMeta(self) -> list[str]:
        return list(self.meta)

    def headings(self) -> list[str]:
        return list(self.head)

    def _index(self, col) -> int:
        if isinstance(col, str):
            if col not in self.head:
                raise ValueError(f"No such column name '{col}' in Results object")
            return self.head.index(col)
        return int(col)

    # results.tpp:36-64
    def column(self, col) -> list:
        i = self._index(col)
        if not self.intcols:
            return []
        nint = len(self.intcols[0])
        if i < nint:
            return [r[i] for r in self.intcols]
        return [r[i - nint] for r in self.fpcols]

    # results.tpp:152-181: sum / nrows (no rows gives nan)
    def mean(self, col) -> float:
        i = self._index(col)
        if not i < len(self.head):
            raise IndexError(f"Index {i} out of range in call to mean")
        vals = self.column(i)
        return sum(vals) / len(vals) if vals else float("nan")

    # results.tpp:183-215: unbiased, sum of squares / (nrows - 1); with no
    # rows the reference divides 0 by SIZE_MAX, with one row 0 by 0
    def variance(self, col) -> float:
        i = self._index(col)
        if not i < len(self.head):
            raise IndexError(f"Index {i} out of range in call to variance")
        vals = self.column(i)
        if not vals:
            return 0.0
        if len(vals) == 1:
            return float("nan")
        m = sum(vals) / len(vals)
        return sum((v - m) ** 2 for v in vals) / (len(vals) - 1)

    # results.tpp:217-268
    def subset(self, cols) -> "Results":
        idx = [self._index(c) for c in cols]
        for i in idx:
            if not i < len(self.head):
                raise IndexError(f"Index {i} is out of range in call to subset")
        out = Results([self.head[i] for i in idx])
        if self.intcols:
            nint = len(self.intcols[0])
            for ri, rf in zip(self.intcols, self.fpcols):
                out.intcols.append([ri[i] for i in idx if i < nint])
                out.fpcols.append([rf[i - nint] for i in idx if i >= nint])
        return out

    @staticmethod
    def _fmt(x) -> str:
        """std::ostream << x with the default flags and precision 6."""
        if isinstance(x, int):
            return str(x)
        if math.isnan(x):
            return "-nan" if math.copysign(1.0, x) < 0 else "nan"
        if math.isinf(x):
            return "-inf" if x < 0 else "inf"
        return "%g" % x

    def _lines(self, sep: str) -> list[str]:
        out = []
        for ri, rf in zip(self.intcols, self.fpcols):
            out.append(sep.join(self._fmt(v) for v in ri + rf))
        return out

    # results.tpp:315-355
    def writeToFile(self, filename: str) -> None:
        if self.intcols and not self.fpcols[0]:
            raise ValueError("a row needs at least one floating point column")
        with open(filename, "w") as f:
            for m in self.meta:
                f.write(f"# {m}\n")
            f.write("\n")
            f.write(" ".join(self.head) + "\n")
            for line in self._lines(" "):
                f.write(line + "\n")

    # results.tpp:271-313
    def print(self) -> None:
        print()
        print("--- META-DATA ---")
        for m in self.meta:
            print(m)
        print()
        print("--- TABLE BODY ---")
        print(", ".join(self.head))
        for line in self._lines(", "):
            print(line)
        print("------------------")
