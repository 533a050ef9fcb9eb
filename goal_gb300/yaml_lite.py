"""Reader for the YAML subset goal's input files use (Teuchos YAML parameter
lists): nested block mappings by indentation, scalars (numbers, quoted or bare
strings, true/false) and flow sequences ``[a, b, c]``; ``#`` comments."""
from __future__ import annotations

from typing import Any, List, Tuple


def _scalar(text: str) -> Any:
    t = text.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low == "true":
        return True
    if low == "false":
        return False
    try:
        if any(c in t for c in ".eE") and not t.lstrip("+-").isdigit():
            return float(t)
        return int(t)
    except ValueError:
        try:
            return float(t)
        except ValueError:
            return t


def _flow_seq(text: str) -> List[Any]:
    inner = text.strip()[1:-1]
    items, cur, q = [], "", None
    for ch in inner:
        if q:
            cur += ch
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur += ch
        elif ch == ",":
            items.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        items.append(cur)
    return [_scalar(x) for x in items]


def _strip_comment(line: str) -> str:
    out, q = "", None
    for ch in line:
        if q:
            out += ch
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out += ch
        elif ch == "#":
            break
        else:
            out += ch
    return out.rstrip()


def loads(text: str) -> dict:
    lines: List[Tuple[int, str]] = []
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip():
            continue
        lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    root: dict = {}
    stack: List[Tuple[int, dict]] = [(-1, root)]
    for indent, content in lines:
        if ":" not in content:
            raise ValueError(f"unsupported YAML line: {content}")
        key, _, rest = content.partition(":")
        key = key.strip()
        while stack and indent <= stack[-1][0]:
            stack.pop()
        parent = stack[-1][1]
        rest = rest.strip()
        if not rest:
            child: dict = {}
            parent[key] = child
            stack.append((indent, child))
        elif rest.startswith("["):
            parent[key] = _flow_seq(rest)
        else:
            parent[key] = _scalar(rest)
    return root


def load(path: str) -> dict:
    with open(path) as f:
        return loads(f.read())
