"""Times the CPU port against the unmodified reference on the same input and
host — TEST INFRASTRUCTURE ONLY (it pins the speed of the CPU baseline that
the benchmark reports, which runs the port where the reference cannot be
built).

    python oracle/speed_check.py [n]

The input is the benchmark's periodic box scaled to n particles (uniform,
seed 1002, about 5 particles per reference block).  The reference times its
own container_periodic::compute_all_cells() (one thread: it has none of its
own; its cells carry no neighbour lists) and the same cells through
compute_cell with voronoicell_neighbor (volume, centroid and neighbours, the
fields the engine computes); the port computes the latter on one thread and
on every host thread.  Prints one JSON line.
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main(n=500_000):
    from oracle import REF_SO, PortLib, RefLib, build_port, build_ref
    from voro_gb300 import workloads as W
    build_port()
    if not build_ref() or not os.path.exists(REF_SO):
        print(json.dumps({"unavailable": "reference sources not present on this host"}))
        return 1
    L = 100.0 * (n / 4_000_000) ** (1.0 / 3.0)
    g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
    w = W.periodic_cube(n=n, L=L, seed=1002, grid=(g, g, g))
    ref = RefLib()
    port = PortLib()
    t_ref, sv = ref.time_compute_all(w)
    t0 = time.perf_counter()
    recs = ref.compute(w)   # compute_cell with voronoicell_neighbor over c_loop_all_periodic
    t_refnb = time.perf_counter() - t0
    t_port1, m1 = port.time_cells(w, threads=1)
    threads = os.cpu_count() or 1
    t_portn, mn = port.time_cells(w, threads=threads)
    print(json.dumps({
        "input": f"container_periodic L={L:.4g}, {n} particles uniform (seed 1002), blocks {g}^3",
        "host": f"{platform.machine()}, {threads} hardware threads",
        "reference_compute_all_cells_1_thread": {"seconds": t_ref, "cells_per_s": n / t_ref,
                                                 "sum_volumes": sv},
        "reference_neighbor_cells_1_thread": {"seconds": t_refnb, "cells_per_s": len(recs) / t_refnb,
                                              "what": "compute_cell(voronoicell_neighbor) per cell, "
                                                      "with volume, centroid and neighbours"},
        "port_1_thread": {"seconds": t_port1, "cells_per_s": m1 / t_port1},
        "port_all_threads": {"threads": threads, "seconds": t_portn, "cells_per_s": mn / t_portn},
        "port_over_reference_1_thread": (m1 / t_port1) / (n / t_ref),
        "port_over_reference_neighbor_1_thread": (m1 / t_port1) / (len(recs) / t_refnb),
    }))
    return 0


if __name__ == "__main__":
    sys.exit(main(int(sys.argv[1]) if len(sys.argv) > 1 else 500_000))
