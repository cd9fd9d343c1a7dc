"""Summaries of Nsight Compute CSV output (the machine-written record of a
capture), in the form the benchmark reads back.

A capture such as

    ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum \\
        --clock-control none -k regex:tc_ --csv --log-file traffic.csv \\
        python bench.py --n 33554432 ...

lists one row per (launch, metric).  ``summarize`` folds the rows per kernel
name: launches, DRAM bytes read and written per launch, device time per
launch, and those bytes divided by the input samples the captured workload
processed per step.  ``write`` stores the result as ``key: value`` lines
(with the command that made the capture) for the benchmark to read with
``read``:

    python -m libfalcon_dsp_gb300.ncu_summary traffic.csv --n-in 33554432 \\
        --steps 2 --out profiles/<kernel>_<workload>_dram.txt --command "<ncu ...>"
"""
from __future__ import annotations

import argparse
import csv
import re

_BYTE_UNITS = {"byte": 1.0, "kbyte": 1e3, "mbyte": 1e6, "gbyte": 1e9, "tbyte": 1e12,
               "kibyte": 1024.0, "mibyte": 1024.0 ** 2, "gibyte": 1024.0 ** 3}
_TIME_UNITS = {"nsecond": 1e-9, "usecond": 1e-6, "msecond": 1e-3, "second": 1.0, "ns": 1e-9, "us": 1e-6,
               "ms": 1e-3, "s": 1.0}


def _value(text: str, unit: str, table: dict) -> float:
    v = float(text.replace(",", ""))
    return v * table.get(unit.strip().lower(), 1.0)


def _short(name: str) -> str:
    """Kernel name without template arguments and parameter list."""
    m = re.match(r"\s*(?:void\s+)?(?:[\w:]+::)?(\w+)", name)
    return m.group(1) if m else name.strip()


def parse(path: str) -> list[dict]:
    """Rows of an ncu --csv log (lines before the header are ncu's own
    messages and the program's output)."""
    with open(path, newline="") as f:
        lines = f.read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.startswith('"ID"'))
    return list(csv.DictReader(lines[start:]))


def summarize(rows: list[dict], n_in: int, steps: int) -> dict:
    """Per kernel: launches, dram bytes/launch, ns/launch; and per step and
    input sample (launches / steps of them make one step)."""
    acc: dict[str, dict] = {}
    for r in rows:
        k = _short(r["Kernel Name"])
        a = acc.setdefault(k, {"ids": set(), "read": 0.0, "write": 0.0, "time": 0.0})
        a["ids"].add(r["ID"])
        m, u, v = r["Metric Name"], r.get("Metric Unit", ""), r["Metric Value"]
        if m == "dram__bytes_read.sum":
            a["read"] += _value(v, u, _BYTE_UNITS)
        elif m == "dram__bytes_write.sum":
            a["write"] += _value(v, u, _BYTE_UNITS)
        elif m == "gpu__time_duration.sum":
            a["time"] += _value(v, u, _TIME_UNITS)
    out = {}
    for k, a in acc.items():
        n = len(a["ids"])
        out[k] = {"launches": n, "dram_read_bytes_per_launch": a["read"] / n,
                  "dram_write_bytes_per_launch": a["write"] / n, "ns_per_launch": 1e9 * a["time"] / n,
                  "dram_bytes_per_input_sample": (a["read"] + a["write"]) / (steps * n_in),
                  "launches_per_step": n / steps}
    return out


def write(summary: dict, path: str, n_in: int, steps: int, command: str, note: str = "") -> None:
    with open(path, "w") as f:
        f.write("# DRAM traffic per kernel from an ncu CSV capture (written by libfalcon_dsp_gb300.ncu_summary)\n")
        f.write(f"command: {command}\n")
        f.write(f"n_in: {n_in}\nsteps: {steps}\n")
        if note:
            f.write(f"note: {note}\n")
        tot = 0.0
        for k in sorted(summary):
            s = summary[k]
            tot += s["dram_bytes_per_input_sample"]
            for key in ("launches", "launches_per_step", "dram_read_bytes_per_launch", "dram_write_bytes_per_launch",
                        "ns_per_launch", "dram_bytes_per_input_sample"):
                f.write(f"{k}.{key}: {s[key]:.6g}\n")
        f.write(f"step.dram_bytes_per_input_sample: {tot:.6g}\n")


def read(path: str) -> dict:
    """key: value lines back into a dict (numbers as float)."""
    d = {}
    with open(path) as f:
        for ln in f:
            if ln.startswith("#") or ":" not in ln:
                continue
            k, v = ln.split(":", 1)
            v = v.strip()
            try:
                d[k.strip()] = float(v)
            except ValueError:
                d[k.strip()] = v
    return d


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("csv")
    ap.add_argument("--n-in", type=int, required=True, help="input samples per step of the captured run")
    ap.add_argument("--steps", type=int, default=1, help="steps the capture covers")
    ap.add_argument("--out", required=True)
    ap.add_argument("--command", required=True, help="the ncu command that wrote the CSV")
    ap.add_argument("--note", default="")
    a = ap.parse_args()
    s = summarize(parse(a.csv), a.n_in, a.steps)
    write(s, a.out, a.n_in, a.steps, a.command, a.note)
    for k, v in sorted(s.items()):
        print(k, {kk: round(vv, 3) for kk, vv in v.items()})


if __name__ == "__main__":
    main()
