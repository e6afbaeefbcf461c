"""PyYAML stand-in: configs for golden generation are written as JSON (a YAML subset)."""
import json


class YAMLError(Exception):
    pass


def safe_load(f):
    text = f.read() if hasattr(f, "read") else f
    return json.loads(text)
