"""Logger with the reference's three metadata sections (wakis/logger.py:14-97).

``grid``, ``solver`` and ``wakeSolver`` are plain dicts; ``save_logs`` writes them as
JSON blocks into ``<results_folder>/wakis.log``.  The solver adds its own performance
entries (cell updates per second, steps, kernel launches) to ``solver``.
"""

import json
import os

import numpy as np


class Logger:
    def __init__(self):
        self.grid = {}
        self.solver = {}
        self.wakeSolver = {}

    def save_logs(self, results_folder=None):
        if results_folder is not None:
            self.wakeSolver["results_folder"] = results_folder
        folder = self.wakeSolver["results_folder"]
        os.makedirs(folder, exist_ok=True)
        logfile = os.path.join(folder, "wakis.log")

        def _convert(obj):
            if isinstance(obj, dict):
                return {k: _convert(v) for k, v in obj.items()}
            if isinstance(obj, (list, tuple)):
                return [_convert(v) for v in obj]
            if isinstance(obj, np.ndarray):
                return obj.tolist()
            if isinstance(obj, np.generic):
                return obj.item()
            try:
                json.dumps(obj)
                return obj
            except Exception:
                return str(obj)

        with open(logfile, "w", encoding="utf-8") as fh:
            fh.write("Simulation Parameters\n")
            fh.write("=====================\n\n")
            for title, data in (("WakeSolver Logs", self.wakeSolver), ("Solver Logs", self.solver),
                                ("Grid Logs", self.grid)):
                fh.write(f"\n## {title} ##\n")
                if not data:
                    fh.write("(empty)\n")
                    continue
                fh.write(json.dumps(_convert(data), indent=2, ensure_ascii=False))
                fh.write("\n")
