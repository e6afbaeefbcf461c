"""YAML configuration loading for the `cupymag` config schema.

The reference loads its config with PyYAML's ``safe_load``
(cupymag/core/config_loader.py:20-46).  PyYAML is not a dependency of this
package, so this module carries a small loader for the subset of YAML that the
config schema uses (examples/example_config.yaml:11-133):

* block mappings nested by indentation, ``key: value`` pairs;
* plain, single- and double-quoted scalars, ``#`` comments;
* flow sequences, nested flow sequences (``[[1,0,0],[0,1,0]]``) and block
  sequences (``- item``);
* YAML 1.1 scalar resolution as PyYAML implements it: ``1.25e+6`` and
  ``10.0e-9`` are floats, but ``1e6`` and ``1.0e6`` (no dot, or an unsigned
  exponent) stay strings; ``yes/no/on/off/true/false`` are booleans;
  ``~``/``null``/empty are None.

JSON documents are valid input too (JSON is a YAML subset and the flow parser
accepts it).
"""
from __future__ import annotations

import re
import warnings
from pathlib import Path
from typing import Any, Dict

__all__ = ["ConfigLoader", "safe_load", "YAMLSubsetError"]


class YAMLSubsetError(ValueError):
    """Raised for input outside the supported YAML subset."""


_INT_RE = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_HEX_RE = re.compile(r"^[-+]?0x[0-9a-fA-F_]+$")
_OCT_RE = re.compile(r"^[-+]?0[0-7_]+$")
_FLOAT_RE = re.compile(
    r"^(?:[-+]?(?:[0-9][0-9_]*)\.[0-9_]*(?:[eE][-+][0-9]+)?"
    r"|\.[0-9_]+(?:[eE][-+][0-9]+)?"
    r"|[-+]?\.(?:inf|Inf|INF)"
    r"|\.(?:nan|NaN|NAN))$"
)
_TRUE = {"yes", "Yes", "YES", "true", "True", "TRUE", "on", "On", "ON"}
_FALSE = {"no", "No", "NO", "false", "False", "FALSE", "off", "Off", "OFF"}
_NULL = {"", "~", "null", "Null", "NULL"}


def _resolve_plain(tok: str) -> Any:
    """Resolve an unquoted scalar the way PyYAML's YAML 1.1 resolver does."""
    s = tok.strip()
    if s in _NULL:
        return None
    if s in _TRUE:
        return True
    if s in _FALSE:
        return False
    if _INT_RE.match(s):
        return int(s.replace("_", ""))
    if _HEX_RE.match(s):
        return int(s.replace("_", ""), 16)
    if _OCT_RE.match(s):
        return int(s.replace("_", ""), 8)
    if _FLOAT_RE.match(s):
        t = s.replace("_", "")
        low = t.lower()
        if low.endswith(".inf"):
            return float("-inf") if t.startswith("-") else float("inf")
        if low == ".nan":
            return float("nan")
        return float(t)
    return s


def _strip_comment(line: str) -> str:
    """Remove a trailing ``#`` comment that is outside quotes."""
    out = []
    quote = None
    prev = " "
    for ch in line:
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
        else:
            if ch in ("'", '"'):
                quote = ch
            elif ch == "#" and prev in (" ", "\t"):
                break
            out.append(ch)
        prev = ch
    return "".join(out).rstrip()


class _Flow:
    """Recursive-descent parser for flow collections and quoted scalars."""

    def __init__(self, text: str):
        self.s = text
        self.i = 0

    def ws(self):
        while self.i < len(self.s) and self.s[self.i] in " \t\r\n":
            self.i += 1

    def parse(self):
        self.ws()
        v = self.value(top=True)
        self.ws()
        if self.i != len(self.s):
            raise YAMLSubsetError(f"trailing characters in {self.s!r}")
        return v

    def value(self, top=False):
        self.ws()
        if self.i >= len(self.s):
            return None
        c = self.s[self.i]
        if c == "[":
            return self.seq()
        if c == "{":
            return self.map()
        if c in ("'", '"'):
            return self.quoted()
        # plain scalar: inside a flow collection stop at , ] }
        j = self.i
        stops = "" if top else ",]}"
        while j < len(self.s) and self.s[j] not in stops:
            if not top and self.s[j] == ":" and j + 1 < len(self.s) and self.s[j + 1] in " \t":
                break
            j += 1
        tok = self.s[self.i:j]
        self.i = j
        return _resolve_plain(tok)

    def quoted(self):
        q = self.s[self.i]
        self.i += 1
        out = []
        while True:
            if self.i >= len(self.s):
                raise YAMLSubsetError("unterminated quoted scalar")
            ch = self.s[self.i]
            if q == "'" and ch == "'":
                if self.i + 1 < len(self.s) and self.s[self.i + 1] == "'":
                    out.append("'")
                    self.i += 2
                    continue
                self.i += 1
                break
            if q == '"' and ch == "\\":
                nxt = self.s[self.i + 1]
                out.append({"n": "\n", "t": "\t", '"': '"', "\\": "\\", "/": "/"}.get(nxt, nxt))
                self.i += 2
                continue
            if q == '"' and ch == '"':
                self.i += 1
                break
            out.append(ch)
            self.i += 1
        return "".join(out)

    def seq(self):
        self.i += 1
        items = []
        self.ws()
        if self.s[self.i] == "]":
            self.i += 1
            return items
        while True:
            items.append(self.value())
            self.ws()
            c = self.s[self.i] if self.i < len(self.s) else ""
            if c == ",":
                self.i += 1
                self.ws()
                if self.i < len(self.s) and self.s[self.i] == "]":
                    self.i += 1
                    return items
                continue
            if c == "]":
                self.i += 1
                return items
            raise YAMLSubsetError(f"bad flow sequence near {self.s[self.i:self.i + 20]!r}")

    def map(self):
        self.i += 1
        out = {}
        self.ws()
        if self.s[self.i] == "}":
            self.i += 1
            return out
        while True:
            self.ws()
            key = self.quoted() if self.s[self.i] in "'\"" else self.value()
            self.ws()
            if self.s[self.i] != ":":
                raise YAMLSubsetError("expected ':' in flow mapping")
            self.i += 1
            out[key] = self.value()
            self.ws()
            c = self.s[self.i]
            self.i += 1
            if c == "}":
                return out
            if c != ",":
                raise YAMLSubsetError("expected ',' or '}' in flow mapping")


def _scalar_or_flow(text: str) -> Any:
    t = text.strip()
    if not t:
        return None
    if t[0] in "[{'\"":
        return _Flow(t).parse()
    return _resolve_plain(t)


def _split_key(content: str):
    """Split ``key: rest`` at the first ': ' (or trailing ':') outside quotes."""
    if content[0] in "'\"":
        f = _Flow(content)
        key = f.quoted()
        rest = content[f.i:].lstrip()
        if not rest.startswith(":"):
            return None
        return key, rest[1:].strip()
    for j, ch in enumerate(content):
        if ch == ":" and (j + 1 == len(content) or content[j + 1] in " \t"):
            return _resolve_plain(content[:j]), content[j + 1:].strip()
    return None


def safe_load(text: str) -> Any:
    """Parse a YAML document of the supported subset into Python objects."""
    stripped = text.strip()
    if stripped.startswith("{") or stripped.startswith("["):
        return _Flow(stripped).parse()
    lines = []
    for raw in text.splitlines():
        if raw.strip() in ("---", "...") or raw.lstrip().startswith("%"):
            continue
        line = _strip_comment(raw.replace("\t", "    "))
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        lines.append((indent, line.strip()))
    if not lines:
        return None
    pos = [0]

    def parse_block(indent):
        if pos[0] >= len(lines):
            return None
        ind, content = lines[pos[0]]
        if content.startswith("- ") or content == "-":
            return parse_seq(ind)
        if _split_key(content) is not None:
            return parse_map(ind)
        pos[0] += 1
        return _scalar_or_flow(content)

    def parse_map(indent):
        out: Dict[Any, Any] = {}
        while pos[0] < len(lines):
            ind, content = lines[pos[0]]
            if ind < indent:
                break
            if ind > indent:
                raise YAMLSubsetError(f"unexpected indentation at {content!r}")
            kv = _split_key(content)
            if kv is None:
                raise YAMLSubsetError(f"expected 'key: value' at {content!r}")
            key, rest = kv
            pos[0] += 1
            if rest == "":
                if pos[0] < len(lines) and (lines[pos[0]][0] > ind or
                                            (lines[pos[0]][0] == ind and lines[pos[0]][1].startswith("-"))):
                    out[key] = parse_block(lines[pos[0]][0])
                else:
                    out[key] = None
            else:
                out[key] = _scalar_or_flow(rest)
        return out

    def parse_seq(indent):
        out = []
        while pos[0] < len(lines):
            ind, content = lines[pos[0]]
            if ind != indent or not (content.startswith("- ") or content == "-"):
                break
            rest = content[1:].strip()
            pos[0] += 1
            if rest == "":
                out.append(parse_block(lines[pos[0]][0]) if pos[0] < len(lines) and lines[pos[0]][0] > ind else None)
            elif _split_key(rest) is not None and rest[0] not in "[{":
                # "- key: value" starts an inline mapping
                sub_indent = ind + 2
                lines.insert(pos[0], (sub_indent, rest))
                out.append(parse_map(sub_indent))
            else:
                out.append(_scalar_or_flow(rest))
        return out

    result = parse_block(lines[0][0])
    if pos[0] != len(lines):
        raise YAMLSubsetError(f"could not parse line {lines[pos[0]][1]!r}")
    return result


class ConfigLoader:
    """Load and validate a CuPyMag YAML config (cupymag/core/config_loader.py:26-84).

    Same behaviour as the reference: a missing file raises FileNotFoundError,
    a syntax error raises ValueError, a missing top-level section only warns,
    ``get`` takes a dot path, and ``get_output_dir`` resolves ``output.directory``
    relative to the config file.
    """

    def __init__(self, config_path):
        self.config_path = Path(config_path)
        self.config = self._load_config()

    def _load_config(self) -> Dict[str, Any]:
        if not self.config_path.exists():
            raise FileNotFoundError(
                f"Configuration file not found: {self.config_path}\n"
                f"Please copy an example config from the examples/ directory."
            )
        try:
            config = safe_load(self.config_path.read_text())
        except (YAMLSubsetError, IndexError) as e:
            raise ValueError(f"Invalid YAML syntax in {self.config_path}: {e}")
        if config is None:
            config = {}
        self._validate_config(config)
        return config

    def _validate_config(self, config: Dict[str, Any]):
        for section in ["physics", "grid", "simulation", "output"]:
            if section not in config:
                warnings.warn(
                    f"Warning: Missing required section: {section}, necessary for micromagnetic simulations.",
                    UserWarning,
                )

    def get(self, key_path: str, default=None):
        value = self.config
        for key in key_path.split("."):
            if isinstance(value, dict) and key in value:
                value = value[key]
            else:
                return default
        return value

    def get_section(self, section: str) -> Dict[str, Any]:
        return self.config.get(section, {})

    def get_output_dir(self):
        output = self.get("output", {}) or {}
        directory = output.get("directory")
        if directory is None:
            return self.config_path.parent.resolve()
        dir_path = Path(directory)
        if dir_path.is_absolute():
            return dir_path
        return (self.config_path.parent / dir_path).resolve()
