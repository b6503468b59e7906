"""Reader and writer of OpenFOAM's ASCII dictionary format (FoamFile).

The reader covers what picFoam cases hold: nested dictionaries, entries
ended by ';', lists in parentheses (items may be words, numbers, strings,
nested lists or `name { ... }` pairs), dimension sets in brackets, quoted
strings, counted lists (`3(1 2 3)`, `List<scalar> 3(...)`) and C/C++
comments.  `#include` lines and `$macro` references are kept as words and not
expanded.

Values: a dictionary is a `Dict` (insertion-ordered `dict`), a list a Python
list, a word a `str`, a number an `int` or `float`, a quoted string a
`Quoted` (a `str`).  An entry with several value tokens (`value uniform 0;`)
is a tuple of them; one token stays itself.
"""
import re

import numpy as np


class Dict(dict):
    """An OpenFOAM dictionary (keyword -> value), in file order."""

    def sub(self, key):
        v = self.get(key)
        return v if isinstance(v, Dict) else Dict()

    def word(self, key, default=None):
        v = self.get(key, default)
        if isinstance(v, tuple):
            v = v[0]
        return v

    def number(self, key, default=None):
        v = self.word(key, default)
        if isinstance(v, (int, float)):
            return float(v)
        return default if v is None else float(v)

    def flag(self, key, default=False):
        v = self.word(key, None)
        if v is None:
            return default
        return str(v).lower() in ("true", "on", "yes", "1")


class Quoted(str):
    """A quoted string of the file."""


class Dimensions(list):
    """A dimension set [kg m s K mol A cd]."""


_TOKEN = re.compile(r'"(?:[^"\\]|\\.)*"|[{}();\[\]]|[^\s{}();\[\]"]+')


def strip_comments(text):
    out, i, n = [], 0, len(text)
    while i < n:
        c = text[i]
        if c == '"':
            j = i + 1
            while j < n and text[j] != '"':
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _atom(tok):
    if tok.startswith('"'):
        return Quoted(tok[1:-1])
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        return tok


class _Parser:
    def __init__(self, text):
        self.toks = _TOKEN.findall(strip_comments(text))
        self.i = 0

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else None

    def take(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def dictionary(self, closing):
        d = Dict()
        while True:
            t = self.peek()
            if t is None:
                # end of file: open dictionaries close here, as OpenFOAM's
                # reader accepts
                return d
            if t == closing:
                self.take()
                return d
            if t == ";":
                self.take()
                continue
            key = _atom(self.take())
            if isinstance(key, str) and key.startswith("#"):
                # directive: keep the rest of the line's tokens up to the next keyword
                d[key] = self.value_tokens(directive=True)
                continue
            if self.peek() == "{":
                self.take()
                d[key] = self.dictionary("}")
            else:
                d[key] = self.value_tokens()
        return d

    def value_tokens(self, directive=False):
        vals = []
        while True:
            t = self.peek()
            if t is None or t == ";" or t == "}":
                if t == ";":
                    self.take()
                break
            if directive and vals:
                break
            vals.append(self.item())
        if len(vals) == 1:
            return vals[0]
        return tuple(vals)

    def item(self):
        t = self.take()
        if t == "(":
            return self.list_body()
        if t == "[":
            dims = Dimensions()
            while self.peek() != "]":
                dims.append(_atom(self.take()))
            self.take()
            return dims
        if t == "{":
            return self.dictionary("}")
        a = _atom(t)
        # counted list "N ( ... )"
        if isinstance(a, int) and self.peek() == "(":
            self.take()
            return self.list_body()
        return a

    def list_body(self):
        items = []
        while True:
            t = self.peek()
            if t is None:
                raise ValueError("unterminated list")
            if t == ")":
                self.take()
                return items
            if t == ";":
                self.take()
                continue
            v = self.item()
            if isinstance(v, str) and self.peek() == "{":
                self.take()
                items.append((v, self.dictionary("}")))
            else:
                items.append(v)


def parse(text):
    """Parse a FoamFile text into a Dict (the FoamFile header included)."""
    return _Parser(text).dictionary(None)


def read(path):
    with open(path) as f:
        return parse(f.read())


# ----------------------------------------------------------------- writer --
_BANNER = """/*--------------------------------*- C++ -*----------------------------------*\\
  =========                 |
  \\\\      /  F ield         | OpenFOAM: The Open Source CFD Toolbox
   \\\\    /   O peration     |
    \\\\  /    A nd           |
     \\\\/     M anipulation  |
\\*---------------------------------------------------------------------------*/
"""


def header(cls, obj, location=None, note=None):
    lines = [_BANNER, "FoamFile\n{\n", "    version     2.0;\n", "    format      ascii;\n",
             f"    class       {cls};\n"]
    if note:
        lines.append(f'    note        "{note}";\n')
    if location is not None:
        lines.append(f'    location    "{location}";\n')
    lines.append(f"    object      {obj};\n}}\n\n")
    return "".join(lines)


def format_scalars(v):
    v = np.asarray(v, dtype=np.float64).ravel()
    return f"{len(v)}\n(\n" + "\n".join("%.17g" % x for x in v) + "\n)\n"


def format_vectors(v):
    v = np.asarray(v, dtype=np.float64).reshape(-1, 3)
    return f"{len(v)}\n(\n" + "\n".join("(%.17g %.17g %.17g)" % tuple(r) for r in v) + "\n)\n"


def format_labels(v):
    v = np.asarray(v, dtype=np.int64).ravel()
    return f"{len(v)}\n(\n" + "\n".join(str(int(x)) for x in v) + "\n)\n"


def numeric_list(v):
    """A parsed list of numbers / 3-vectors as a numpy array."""
    if isinstance(v, tuple):
        v = [x for x in v if isinstance(x, list)][-1]
    return np.asarray(v, dtype=np.float64)
