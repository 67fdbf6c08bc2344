"""Saved launch tuning: the autotuner's choice for a device and workload.

ncg_autotune (include/ncg.h) searches the NCG_TUNE_* keys on a batch and
leaves the fastest values in the context.  This module keeps those values in
a small JSON file keyed by device name, SM count and a workload name, so that
later runs apply them without searching again.  Results never depend on the
tuning; only the launch configuration does.
"""
from __future__ import annotations

import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PATH = os.path.join(HERE, "tuning", "gb300.json")


def _key(device_name, sms, workload):
    return f"{device_name}|{int(sms)}|{workload}"


def load(path=DEFAULT_PATH):
    """All saved entries ({} when the file does not exist)."""
    try:
        with open(path) as f:
            return json.load(f)
    except FileNotFoundError:
        return {}


def lookup(device_name, sms, workload, path=DEFAULT_PATH):
    """The saved {key name: value} for this device and workload, or None."""
    e = load(path).get(_key(device_name, sms, workload))
    return None if e is None else dict(e["values"])


def save(device_name, sms, workload, values, ms=None, extra=None, path=DEFAULT_PATH):
    """Adds or replaces the entry for this device and workload."""
    data = load(path)
    entry = {"values": {k: int(v) for k, v in values.items()}}
    if ms is not None:
        entry["ms"] = float(ms)
    if extra:
        entry.update(extra)
    data[_key(device_name, sms, workload)] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    os.replace(tmp, path)
    return entry
