"""Minimal reader for Rusty Object Notation (RON), enough for SyFrack's graph,
scene and fixture files (crates/syfrack-core/src/scene/graph/bundled.rs loads
graphs/*.ron with the ron 0.12 crate; this module reads the same text).

Values map to Python as follows:
  (a: 1, b: 2)      -> dict (struct; anonymous or named, name in key "__name__")
  Name(a: 1)        -> dict with "__name__": "Name"
  Name(1, 2) / (1,2)-> Tuple(name, items)
  Name              -> Unit("Name")  (unit variant / unit struct)
  [1, 2]            -> list
  "text"            -> str, numbers -> int/float, true/false -> bool, None / Some(x)
"""
from __future__ import annotations

import re
from dataclasses import dataclass
from typing import Any


class RonError(ValueError):
    pass


@dataclass(frozen=True)
class Unit:
    name: str


@dataclass
class Tuple:
    name: str | None
    items: list


_NUM = re.compile(r"[+-]?(?:inf|NaN|(?:\d[\d_]*(?:\.[\d_]*)?|\.\d[\d_]*)(?:[eE][+-]?\d+)?)")
# an identifier, or a raw one (r#name: the name itself, never a keyword such as None)
_IDENT = re.compile(r"(?:r#)?[A-Za-z_][A-Za-z0-9_]*")


class _Parser:
    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def ws(self):
        s, n = self.s, len(self.s)
        while self.i < n:
            c = s[self.i]
            if c in " \t\r\n,":
                # commas are separators; trailing commas are legal in RON
                if c == ",":
                    return
                self.i += 1
            elif s.startswith("//", self.i):
                j = s.find("\n", self.i)
                self.i = n if j < 0 else j + 1
            elif s.startswith("/*", self.i):
                j = s.find("*/", self.i)
                if j < 0:
                    raise RonError("unterminated block comment")
                self.i = j + 2
            elif s.startswith("#![", self.i):
                j = s.find("]", self.i)
                self.i = j + 1
            else:
                return

    def skip(self):
        while True:
            self.ws()
            if self.i < len(self.s) and self.s[self.i] == ",":
                self.i += 1
                continue
            return

    def peek(self) -> str:
        self.ws()
        return self.s[self.i] if self.i < len(self.s) else ""

    def expect(self, ch: str):
        self.ws()
        if not self.s.startswith(ch, self.i):
            raise RonError(f"expected {ch!r} at {self.i}: {self.s[self.i:self.i + 30]!r}")
        self.i += len(ch)

    def value(self) -> Any:
        c = self.peek()
        if c == "":
            raise RonError("unexpected end of input")
        if c == "(":
            return self.parens(None)
        if c == "[":
            return self.list_()
        if c == '"':
            return self.string()
        if c == "'":
            j = self.s.index("'", self.i + 1)
            v = self.s[self.i + 1:j]
            self.i = j + 1
            return v
        m = _NUM.match(self.s, self.i)
        if m and (c in "+-.0123456789" or m.group(0) in ("inf", "NaN")):
            if c not in "+-.0123456789" and self.s[m.end():m.end() + 1].isalnum():
                m = None
        if m and m.group(0):
            txt = m.group(0).replace("_", "")
            self.i = m.end()
            if txt in ("inf", "+inf"):
                return float("inf")
            if txt == "-inf":
                return float("-inf")
            if txt == "NaN":
                return float("nan")
            if re.fullmatch(r"[+-]?\d+", txt):
                return int(txt)
            return float(txt)
        m = _IDENT.match(self.s, self.i)
        if not m:
            raise RonError(f"unexpected {self.s[self.i:self.i + 20]!r} at {self.i}")
        name = m.group(0)
        self.i = m.end()
        if name.startswith("r#"):
            name = name[2:]
            if self.i < len(self.s) and self.s[self.i] == "(":
                return self.parens(name)
            return Unit(name)
        if name == "true":
            return True
        if name == "false":
            return False
        if name == "None":
            return None
        if self.i < len(self.s) and self.s[self.i] == "(":
            if name == "Some":
                self.expect("(")
                v = self.value()
                self.skip()
                self.expect(")")
                return v
            return self.parens(name)
        return Unit(name)

    def string(self) -> str:
        self.expect('"')
        out = []
        s = self.s
        while True:
            c = s[self.i]
            if c == '"':
                self.i += 1
                return "".join(out)
            if c == "\\":
                e = s[self.i + 1]
                if e == "u":
                    if s[self.i + 2] == "{":
                        j = s.index("}", self.i)
                        out.append(chr(int(s[self.i + 3:j], 16)))
                        self.i = j + 1
                        continue
                    out.append(chr(int(s[self.i + 2:self.i + 6], 16)))
                    self.i += 6
                    continue
                out.append({"n": "\n", "t": "\t", "r": "\r", "0": "\0"}.get(e, e))
                self.i += 2
                continue
            out.append(c)
            self.i += 1

    def list_(self) -> list:
        self.expect("[")
        items = []
        while True:
            self.skip()
            if self.peek() == "]":
                self.i += 1
                return items
            items.append(self.value())

    def parens(self, name: str | None):
        self.expect("(")
        # struct if the first token is "ident:" (and not "ident::")
        self.skip()
        m = _IDENT.match(self.s, self.i)
        is_struct = False
        if m:
            j = m.end()
            while j < len(self.s) and self.s[j] in " \t\r\n":
                j += 1
            if j < len(self.s) and self.s[j] == ":" and not self.s.startswith("::", j):
                is_struct = True
        if self.peek() == ")":
            self.i += 1
            return {"__name__": name} if name else Tuple(None, [])
        if is_struct:
            d: dict = {"__name__": name} if name else {}
            while True:
                self.skip()
                if self.peek() == ")":
                    self.i += 1
                    return d
                m = _IDENT.match(self.s, self.i)
                if not m:
                    raise RonError(f"expected field name at {self.i}")
                self.i = m.end()
                self.expect(":")
                d[m.group(0).removeprefix("r#")] = self.value()
        items = []
        while True:
            self.skip()
            if self.peek() == ")":
                self.i += 1
                return Tuple(name, items)
            items.append(self.value())


def loads(text: str) -> Any:
    p = _Parser(text)
    v = p.value()
    p.skip()
    if p.i < len(p.s) and p.s[p.i:].strip():
        raise RonError(f"trailing data at {p.i}")
    return v


def load(path) -> Any:
    with open(path, encoding="utf-8") as f:
        return loads(f.read())


def vec(v) -> list[float]:
    """A glam Vec3/Vec2 or array written as a RON tuple or list."""
    if isinstance(v, Tuple):
        return [float(x) for x in v.items]
    if isinstance(v, (list, tuple)):
        return [float(x) for x in v]
    raise RonError(f"not a vector: {v!r}")
