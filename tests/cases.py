"""Seeded small cases shared by the tests (sizes the oracle finishes in seconds)."""
import __graft_entry__ as ge

wl = ge.load_package().workload


def small_cases():
    """(label, Case) pairs covering flat tank, beach + obstacles + partial cells,
    a bore front (x-oriented surface cells, corner cells) and a shoreline."""
    return [
        ("tank_24x20x16", wl.make_case(24, 20, 16, dz=0.025, partial=False, seed=0, eps0=1e-12)),
        ("beach_48x40x24", wl.beach_case(48, 40, 24, seed=5, n_obstacles=6)),
        ("bore_40x24x32", wl.make_case(40, 24, 32, dz=0.8 / 32, slope=0.5, n_obstacles=4, seed=7,
                                        amplitude=0.08, step_layers=2)),
        ("bore3_40x24x32", wl.make_case(40, 24, 32, dz=0.8 / 32, slope=None, n_obstacles=4, seed=8,
                                         amplitude=0.08, step_layers=3)),
        ("shore_64x16x24", wl.make_case(64, 16, 24, slope=1.0 / 3.0, n_obstacles=3, seed=11,
                                         amplitude=0.05)),
    ]
