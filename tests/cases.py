"""Small hand-made and seeded inputs shared by the tests."""
import numpy as np


def a(rows):
    return np.asarray(rows, np.float32).reshape(-1, 4)


def hand_cases():
    """Edge cases the reference code paths meet: empty, single, pairs, triplets,
    collinear and tangent configurations, a tetrahedron and a small cluster."""
    s3 = np.sqrt(3.0)
    cases = {
        "empty": a([]),
        "single": a([[0, 0, 0, 1.7]]),
        "pair": a([[0, 0, 0, 1.7], [2.5, 0, 0, 1.5]]),
        "pair_far": a([[0, 0, 0, 1.7], [20, 0, 0, 1.5]]),
        "triangle": a([[0, 0, 0, 1.7], [3.0, 0, 0, 1.7], [1.5, 2.6, 0, 1.7]]),
        "collinear": a([[0, 0, 0, 1.7], [2.0, 0, 0, 1.7], [4.0, 0, 0, 1.7]]),
        "tangent": a([[0, 0, 0, 1.6], [6.0, 0, 0, 1.6]]),  # SAS spheres touch (R = 3.0 each)
        "tetrahedron": a([[1, 1, 1, 1.7], [1, -1, -1, 1.55], [-1, 1, -1, 1.52], [-1, -1, 1, 1.8]]) * np.float32([2, 2, 2, 1]),
        "square": a([[0, 0, 0, 1.7], [3.4, 0, 0, 1.7], [0, 3.4, 0, 1.7], [3.4, 3.4, 0, 1.7]]),
        "hexring": a([[3.2 * np.cos(t), 3.2 * np.sin(t), 0, 1.7] for t in np.arange(6) * np.pi / 3]),
        "octahedron": a([[3, 0, 0, 1.7], [-3, 0, 0, 1.7], [0, 3, 0, 1.7], [0, -3, 0, 1.7], [0, 0, 3, 1.7],
                         [0, 0, -3, 1.7]]),
        "stack": a([[0, 0, 1.6 * k, 1.7] for k in range(8)]),
        "trigonal": a([[0, 0, 0, 1.8], [3.1, 0, 0, 1.6], [-1.55, 3.1 * s3 / 2, 0, 1.6], [-1.55, -3.1 * s3 / 2, 0, 1.6],
                       [0, 0, 3.0, 1.5]]),
    }
    rng = np.random.default_rng(7)
    pts = rng.uniform(-6, 6, (40, 3))
    cases["cluster40"] = a(np.c_[pts, rng.choice([1.52, 1.55, 1.7, 1.8], 40)])
    return cases
