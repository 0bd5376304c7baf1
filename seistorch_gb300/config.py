"""Configuration loading for the YAML schema of seistorch (template.yml).

PyYAML is used when importable; otherwise a small reader handles the subset
the configs use (nested mappings by indentation, ``- item`` lists including
nested ``- - a`` lists, scalars, ``~``/empty as None, inline ``[a, b]``).
"""
import json
import os


def _scalar(s):
    s = s.strip()
    if s in ("", "~", "null", "None"):
        return None
    if s in ("true", "True"):
        return True
    if s in ("false", "False"):
        return False
    if (s[0] == s[-1]) and s[0] in "'\"" and len(s) >= 2:
        return s[1:-1]
    if s.startswith("[") and s.endswith("]"):
        inner = s[1:-1].strip()
        return [] if not inner else [_scalar(p) for p in inner.split(",")]
    try:
        return int(s)
    except ValueError:
        pass
    try:
        return float(s)
    except ValueError:
        return s


def _strip_comment(line):
    out, q = [], None
    for ch in line:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def _parse(lines, i, indent):
    """Parse a block whose lines are indented >= indent, starting at i."""
    if i < len(lines) and lines[i][1].startswith("- "):
        return _parse_list(lines, i, indent)
    out = {}
    while i < len(lines):
        ind, text = lines[i]
        if ind < indent:
            break
        if text.startswith("- "):
            break
        key, _, rest = text.partition(":")
        key = key.strip()
        rest = rest.strip()
        i += 1
        if rest:
            out[key] = _scalar(rest)
        elif i < len(lines) and (lines[i][0] > ind or (lines[i][0] == ind and lines[i][1].startswith("- "))):
            out[key], i = _parse(lines, i, lines[i][0])
        else:
            out[key] = None
    return out, i


def _parse_list(lines, i, indent):
    out = []
    while i < len(lines):
        ind, text = lines[i]
        if ind != indent or not text.startswith("- "):
            break
        item = text[2:].strip()
        i += 1
        if item.startswith("- "):
            # nested list: re-read the item as a list at a deeper indent
            sub = [(ind + 2, item)]
            while i < len(lines) and lines[i][0] > ind:
                sub.append(lines[i])
                i += 1
            val, _ = _parse_list(sub, 0, ind + 2)
            out.append(val)
        elif ":" in item and not item.startswith(("'", '"')):
            sub = [(ind + 2, item)]
            while i < len(lines) and lines[i][0] > ind:
                sub.append(lines[i])
                i += 1
            val, _ = _parse(sub, 0, ind + 2)
            out.append(val)
        else:
            out.append(_scalar(item))
    return out, i


def loads(text):
    lines = []
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip():
            continue
        lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    if not lines:
        return {}
    val, _ = _parse(lines, 0, lines[0][0])
    return val


def read_cfg(path):
    """Load a YAML (or JSON) config file into a dict (io.py:333-350)."""
    with open(path) as f:
        text = f.read()
    if path.endswith(".json"):
        return json.loads(text)
    try:
        import yaml  # noqa: F401
        return yaml.safe_load(text)
    except ImportError:
        return loads(text)


def load_config(cfg):
    if isinstance(cfg, dict):
        import copy
        return copy.deepcopy(cfg)
    if isinstance(cfg, (str, os.PathLike)):
        return read_cfg(str(cfg))
    raise TypeError("config must be a dict or a path")
