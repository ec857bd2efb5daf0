"""CPU tests of the synthetic workloads' shapes: the uneven batch spans the
configuration sizes and neighbour counts it is meant to (16-432 atoms,
about 20-70 neighbours, with atoms that need a second 64-bond tile)."""
from __future__ import annotations

import numpy as np


def test_uneven_batch_spans_sizes_and_neighbour_counts():
    from magace import structures as S
    confs = S.uneven_batch(256, seed=3)
    sizes = [len(c.positions) for c in confs]
    assert min(sizes) >= 16 and max(sizes) == 432
    counts = np.concatenate([(lambda nb: nb.nstop - nb.nstart + 1)(S.neighbor_data(c, 5.0)) for c in confs])
    assert counts.min() <= 24 and counts.max() >= 66
    assert (counts > 64).sum() >= 50  # atoms whose bonds span two 64-bond tiles
