"""A small YAML reader for telescope configuration files.

Covers the subset the configuration schema uses: block mappings, block
sequences ("- " items, including mappings and nested sequences inside
them), flow sequences on one line ("[1, 2]", "[]"), plain and quoted
scalars, comments. Numbers become int/float, true/false/null their Python
values, everything else a string. PyYAML, when installed, is not needed.
"""
from __future__ import annotations

import re

_INT = re.compile(r"^[-+]?\d+$")
_FLOAT = re.compile(r"^[-+]?(\d+\.\d*|\.\d+|\d+)([eE][-+]?\d+)?$|^[-+]?\.(inf|Inf|INF)$|^\.(nan|NaN|NAN)$")


def _scalar(tok: str):
    t = tok.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if (t[0] == t[-1]) and t[0] in "'\"" and len(t) >= 2:
        return t[1:-1]
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        low = t.lower()
        if low.endswith("inf"):
            return float("-inf") if low.startswith("-") else float("inf")
        if low.endswith("nan"):
            return float("nan")
        return float(t)
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [] if not inner else [_scalar(p) for p in _split_flow(inner)]
    if t == "{}":
        return {}
    return t


def _split_flow(s: str):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return out


def _strip_comment(line: str) -> str:
    q = None
    for i, ch in enumerate(line):
        if ch in "'\"":
            q = None if q == ch else (ch if q is None else q)
        elif ch == "#" and q is None and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _lines(text: str):
    out = []
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        out.append((len(line) - len(line.lstrip(" ")), line.strip()))
    return out


class _Parser:
    def __init__(self, lines):
        self.lines = lines
        self.i = 0

    def parse(self, indent: int):
        if self.i >= len(self.lines):
            return None
        ind, text = self.lines[self.i]
        if text.startswith("- ") or text == "-":
            return self.seq(ind)
        return self.mapping(ind)

    def mapping(self, indent: int):
        out = {}
        while self.i < len(self.lines):
            ind, text = self.lines[self.i]
            if ind < indent or text.startswith("- ") or text == "-":
                if ind < indent or ind == indent:
                    break
            if ind != indent:
                raise ValueError(f"bad indentation at line {self.i}: {text!r}")
            key, _, rest = text.partition(":")
            key = key.strip().strip("'\"")
            rest = rest.strip()
            self.i += 1
            if rest:
                out[key] = _scalar(rest)
            elif self.i < len(self.lines) and (self.lines[self.i][0] > indent or
                                               (self.lines[self.i][0] == indent and
                                                self.lines[self.i][1].startswith("-"))):
                out[key] = self.parse(self.lines[self.i][0])
            else:
                out[key] = None
        return out

    def seq(self, indent: int):
        out = []
        while self.i < len(self.lines):
            ind, text = self.lines[self.i]
            if ind != indent or not (text.startswith("- ") or text == "-"):
                break
            body = text[1:].strip()
            if not body:
                self.i += 1
                out.append(self.parse(self.lines[self.i][0]) if self.i < len(self.lines) and
                           self.lines[self.i][0] > indent else None)
            elif body.startswith("- "):
                # nested sequence starting on the same line: re-indent it
                self.lines[self.i] = (indent + 2, body)
                out.append(self.seq(indent + 2))
            elif ":" in body and not body.startswith(("'", '"', "[")) and re.match(r"^[^:\[\]]+:(\s|$)", body):
                self.lines[self.i] = (indent + 2, body)
                out.append(self.mapping(indent + 2))
            else:
                self.i += 1
                out.append(_scalar(body))
        return out


def safe_load(text_or_file):
    text = text_or_file.read() if hasattr(text_or_file, "read") else text_or_file
    lines = _lines(text)
    if not lines:
        return None
    return _Parser(lines).parse(lines[0][0])
