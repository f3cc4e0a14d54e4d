"""A small YAML reader for OpenPixi input decks (no third-party YAML package).

The reference reads its decks with snakeyaml into public fields
(ui/util/yaml/YamlParser.java:15-19, YamlSettings.java).  The decks use block
mappings, block sequences (of mappings or scalars), flow sequences of scalars
(``gridCells: [128, 32, 32]``), ``#`` comments and plain or quoted scalars; that
subset is what this reader accepts.  Anything else raises ``ValueError``.
"""
import re

_INT = re.compile(r"^[-+]?\d+$")
_FLOAT = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")


def _scalar(tok):
    t = tok.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        return float(t)
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [] if not inner else [_scalar(x) for x in _split_flow(inner)]
    return t


def _split_flow(s):
    out, depth, cur, q = [], 0, "", None
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "[":
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


def _strip_comment(line):
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _lines(text):
    out = []
    for raw in text.splitlines():
        if raw.strip() in ("---", "..."):
            continue
        s = _strip_comment(raw).rstrip()
        if not s.strip():
            continue
        if "\t" in s[: len(s) - len(s.lstrip())]:
            raise ValueError("tabs are not allowed for indentation")
        out.append((len(s) - len(s.lstrip(" ")), s.strip()))
    return out


def _parse_block(lines, i, indent):
    """Parse the block starting at lines[i] with the given indentation."""
    if i >= len(lines):
        return None, i
    ind, text = lines[i]
    if text.startswith("- ") or text == "-":
        seq = []
        while i < len(lines) and lines[i][0] == indent and (lines[i][1].startswith("- ") or lines[i][1] == "-"):
            item = lines[i][1][1:].strip()
            if not item:
                val, i = _parse_block(lines, i + 1, lines[i + 1][0] if i + 1 < len(lines) else indent + 2)
                seq.append(val)
                continue
            if _is_key(item):
                # mapping inside a sequence item: first key on the dash line
                sub_indent = indent + 2
                fake = [(sub_indent, item)]
                j = i + 1
                while j < len(lines) and lines[j][0] > indent:
                    fake.append(lines[j])
                    j += 1
                val, _ = _parse_block(fake, 0, sub_indent)
                seq.append(val)
                i = j
            else:
                seq.append(_scalar(item))
                i += 1
        return seq, i
    mapping = {}
    while i < len(lines) and lines[i][0] == indent:
        text = lines[i][1]
        if not _is_key(text):
            raise ValueError(f"expected 'key: value', got {text!r}")
        key, rest = text.split(":", 1)
        key = key.strip().strip("'\"")
        rest = rest.strip()
        if rest:
            mapping[key] = _scalar(rest)
            i += 1
        else:
            if i + 1 < len(lines) and (lines[i + 1][0] > indent or
                                       (lines[i + 1][0] == indent and lines[i + 1][1].startswith("-"))):
                val, i = _parse_block(lines, i + 1, lines[i + 1][0])
                mapping[key] = val
            else:
                mapping[key] = None
                i += 1
    if i < len(lines) and lines[i][0] > indent:
        raise ValueError(f"bad indentation at {lines[i][1]!r}")
    return mapping, i


def _is_key(text):
    m = re.match(r"^(\"[^\"]*\"|'[^']*'|[^:\[\]{}]+):(\s|$)", text)
    return m is not None


def loads(text):
    lines = _lines(text)
    if not lines:
        return {}
    val, i = _parse_block(lines, 0, lines[0][0])
    if i != len(lines):
        raise ValueError(f"unparsed content at {lines[i][1]!r}")
    return val


def load(path):
    with open(path) as f:
        return loads(f.read())
