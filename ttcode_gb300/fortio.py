"""Fortran list-directed input (``READ(u,*)``), the subset ttcode's text
files need: blank or comma separators, null values (two commas), ``r*c``
repeat counts, a slash ending a read, D and Q exponents and exponents
written without a letter; a read continues over records until its items
are filled and drops the rest of its last record; a blank record gives no
value.  Used for the opacity tables (READBURROWSOPCTABLE, pprphy.f:1231)
and the ASCII restart file (READRESTART, ppinit.f:1599-1632).
"""
from __future__ import annotations

import re


class ListDirectedError(ValueError):
    """Input a Fortran list-directed read would stop on."""


_NULL = object()
_SLASH = object()
_EXP = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+))([+-]\d+)$")


def _tokens(record: str):
    """Values of one record: strings, _NULL for an empty value between
    commas, _SLASH for a slash (which ends the read)."""
    out, i, n = [], 0, len(record)
    after_value = False
    while True:
        while i < n and record[i] in " \t":
            i += 1
        if i >= n:
            break
        ch = record[i]
        if ch == ",":
            if not after_value:
                out.append(_NULL)
            after_value = False
            i += 1
            continue
        if ch == "/":
            out.append(_SLASH)
            break
        if ch in "'\"":
            j, s = i + 1, []
            while j < n:
                if record[j] == ch:
                    if j + 1 < n and record[j + 1] == ch:
                        s.append(ch)
                        j += 2
                        continue
                    break
                s.append(record[j])
                j += 1
            out.append("".join(s))
            i = j + 1
        else:
            j = i
            while j < n and record[j] not in " \t,/":
                j += 1
            tok = record[i:j]
            m = re.match(r"^(\d+)\*(.*)$", tok)
            if m:
                reps, val = int(m.group(1)), m.group(2)
                out.extend([val if val else _NULL] * reps)
            else:
                out.append(tok)
            i = j
        after_value = True
    return out


def real(tok: str) -> float:
    """A REAL or DOUBLE PRECISION item."""
    t = tok.translate(str.maketrans("dDqQ", "eeee"))
    try:
        return float(t)
    except ValueError:
        m = _EXP.match(t)
        if not m:
            raise ValueError(f"not a real number: {tok!r}") from None
        return float(f"{m.group(1)}e{m.group(2)}")


def integer(tok: str) -> int:
    """An INTEGER item."""
    return int(tok)


class ListDirected:
    """Sequential list-directed reads over the records of a text file;
    ``error`` is the exception class raised at the end of the file or on an
    item that does not convert."""

    def __init__(self, lines, name: str = "<file>", error=ListDirectedError):
        self.lines = list(lines)
        self.pos = 0
        self.name = name
        self.error = error

    def _record(self):
        if self.pos >= len(self.lines):
            raise self.error(f"{self.name}: end of file at record {self.pos + 1}")
        rec = self.lines[self.pos].rstrip("\r\n")
        self.pos += 1
        return rec

    def read(self, n: int, conv=real):
        """Up to n values; None where the input gave a null value or a slash
        ended the read (the Fortran variable keeps its value there).
        ``conv`` converts every item, or is a sequence of one converter per
        item (a READ of mixed types)."""
        convs = conv if isinstance(conv, (list, tuple)) else None
        vals = []
        while len(vals) < n:
            toks = _tokens(self._record())
            for t in toks:
                if t is _SLASH:
                    return vals + [None] * (n - len(vals))
                if t is _NULL:
                    vals.append(None)
                else:
                    f = convs[len(vals)] if convs else conv
                    try:
                        vals.append(f(t))
                    except ValueError as e:
                        raise self.error(f"{self.name}, record {self.pos}: {e}") from None
                if len(vals) == n:
                    break
        return vals

    def skip(self):
        """A READ with no items: the next record is passed over."""
        self._record()

    def read_text(self, length: int = 20) -> str:
        """One character item (``character text*20``); a blank record
        counts as no value, so the read moves on to the next record."""
        v = self.read(1, conv=str)[0]
        return "" if v is None else v[:length]
