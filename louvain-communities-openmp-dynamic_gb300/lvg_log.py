"""Log lines of the experiment driver, and their CSV form.

The reference's driver prints one line per run (main.cxx:77-85) and its
``process.js`` turns a log of such lines into a CSV table (process.js:9-92).
``louvain_gb300_experiment`` prints the same lines; this module formats them
(:func:`result_line`) and converts a log into the same CSV rows and columns
(:func:`read_log`, :func:`write_csv`)::

    python lvg_log.py run.log out.csv
"""
from __future__ import annotations

import re
import sys

ROMPTH = re.compile(r"^OMP_NUM_THREADS=(\d+)")
RGRAPH = re.compile(r"^Loading graph .*/(.*?)\.txt \.\.\.", re.M)
RORDER = re.compile(r"^order: (\d+) size: (\d+) (?:\[\w+\] )?\{\}", re.M)
RBATCH = re.compile(r"^order: (\d+) size: (\d+) \[directed\] \{\} \(insertions=(\d+)\)", re.M)
RRESLT = re.compile(r"^\{-(.+?)/\+(.+?) batchf, (.+?) threads\} -> \{(.+?)ms, (.+?)ms mark, (.+?)ms init, "
                    r"(.+?)ms firstpass, (.+?)ms locmove, (.+?)ms aggr, (.+?) aff, (.+?) iters, (.+?) passes, "
                    r"(.+?) modularity\} (.+)", re.M)
RSTAMP = re.compile(r"^\d+-\d+-\d+ \d+:\d+:\d+ ")

RESULT_FIELDS = ["batch_deletions_fraction", "batch_insertions_fraction", "num_threads", "time", "marking_time",
                 "initialization_time", "first_pass_time", "local_moving_phase_time", "aggregation_phase_time",
                 "affected_vertices", "iterations", "passes", "modularity"]


def result_line(r: dict, technique: str, threads: int, modularity: float, deletions_f: float = 0.0,
                insertions_f: float = 0.0) -> str:
    """One result line in main.cxx's format; r holds LouvainResult's scalar fields."""
    return ("{-%.3e/+%.3e batchf, %03d threads} -> {%09.1fms, %09.1fms mark, %09.1fms init, %09.1fms firstpass, "
            "%09.1fms locmove, %09.1fms aggr, %.3e aff, %04d iters, %03d passes, %01.9f modularity} %s" % (
                deletions_f, insertions_f, threads, r["time"], r["markingTime"], r["initializationTime"],
                r["firstPassTime"], r["localMoveTime"], r["aggregationTime"], float(r["affectedVertices"]),
                r["iterations"], r["passes"], modularity, technique))


def _read_line(ln: str, data: dict, state: dict) -> dict:
    ln = RSTAMP.sub("", ln)
    if ROMPTH.search(ln):
        state["omp_num_threads"] = float(ROMPTH.search(ln).group(1))
    elif RGRAPH.search(ln):
        g = RGRAPH.search(ln).group(1)
        data.setdefault(g, [])
        state["graph"] = g
    elif RBATCH.search(ln):
        m = RBATCH.search(ln)
        state["order"], state["size"] = float(m.group(1)), float(m.group(2))
        state["batch_deletions_fraction"] = 0
        state["batch_insertions_fraction"] = 0
        state["batch_index"] = state.get("batch_index", 0) + 1
    elif RORDER.search(ln):
        m = RORDER.search(ln)
        state["order"], state["size"] = float(m.group(1)), float(m.group(2))
        state["batch_deletions_fraction"] = 0
        state["batch_insertions_fraction"] = 0
        state["batch_index"] = -1
    elif RRESLT.search(ln):
        m = RRESLT.search(ln)
        row = dict(state)
        for k, v in zip(RESULT_FIELDS, m.groups()[:13]):
            row[k] = float(v)
        row["technique"] = m.group(14)
        data[state["graph"]].append(row)
    return state


def read_log(path: str) -> dict:
    """Rows of a log, grouped by graph, as process.js's readLog builds them."""
    data: dict = {}
    state: dict = {}
    with open(path) as f:
        for ln in f.read().replace("\r\n", "\n").split("\n"):
            state = _read_line(ln, data, state)
    return data


def rows_of(data: dict) -> list[dict]:
    return [r for rows in data.values() for r in rows]


def write_csv(path: str, rows: list[dict]) -> None:
    """Header of the first row's keys, then every value quoted (process.js writeCsv)."""
    if not rows:
        open(path, "w").close()
        return
    cols = list(rows[0].keys())
    with open(path, "w") as f:
        f.write(",".join(cols) + "\n")
        for r in rows:
            f.write(",".join('"%s"' % _fmt(r.get(c, "")) for c in cols) + "\n")


def _fmt(v) -> str:
    if isinstance(v, float) and v.is_integer():
        return str(int(v))
    return str(v)


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit("usage: python lvg_log.py <log> <csv>")
    write_csv(sys.argv[2], rows_of(read_log(sys.argv[1])))
