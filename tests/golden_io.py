"""Loads the committed golden vectors (tests/golden/vectors.json)."""
import json
import os

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vectors.json")


def load():
    with open(_PATH) as f:
        return json.load(f)
