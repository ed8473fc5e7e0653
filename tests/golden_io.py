"""Loads the committed golden vectors (tests/golden/vectors.json and
tests/golden/ed25519_raw.json)."""
import json
import os

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vectors.json")


def load():
    with open(_PATH) as f:
        return json.load(f)


def load_raw():
    """ed25519 over messages of any length (tests/golden/make_golden_raw.py)."""
    with open(os.path.join(os.path.dirname(_PATH), "ed25519_raw.json")) as f:
        return json.load(f)["ed25519_raw"]
