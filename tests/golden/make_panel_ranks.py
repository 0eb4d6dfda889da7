"""Record the (a, b, c) ranks of the 1953 panel-0 Schur updates of the
65,536-point benchmark panel (2D, exp(-|x-y|^2/0.01), nb 1024, tiles at
1e-8 relative, maxrank 128), as built by hcore_gb300.panel.build_panel on
the host cores.  The sharding test balances these.

    python tests/golden/make_panel_ranks.py   # writes panel_ranks.json here
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    from hcore_gb300 import panel as pnl

    p = pnl.build_panel(device="cpu")
    rows = [[int(p.rank[p.index[(i, 0)]]), int(p.rank[p.index[(j, 0)]]),
             int(p.rank[p.index[(i, j)]])] for i, j in p.updates]
    with open(os.path.join(HERE, "panel_ranks.json"), "w") as f:
        json.dump({"nb": p.nb, "updates": [list(u) for u in p.updates], "abc": rows}, f,
                  separators=(",", ":"))


if __name__ == "__main__":
    main()
