"""Critical points: the C restatement in the oracle against a literal
simulation of the reference critPoints kernel (src/alg/critPoints.cu:49-331)
and against known answers.

The simulation follows the kernel thread by thread on a padded VV (rows of
width max_VV, -1 padding, as VV_kernel + cudaMemset(-1) leave it), with
duplicate entries planted in some rows the way the racy VV_kernel produces
them (cuda_extraction.cu:983-999): execution masks (:85-111), class -1/+1
with the id tie-break (:136-140), the bounded min-label propagation loop
(:170-266), root counting into classes[3v + (class+1)/2] (:275-284) and the
class code (:303-330)."""
import numpy as np
import pytest

from tetragpu_gb300 import meshgen


def simulate_reference_kernel(vv_rows, field, rng=None):
    V = len(vv_rows)
    max_appear = max((len(r) for r in vv_rows), default=1)
    max_vv = max(32, ((3 * max_appear + 31) // 32) * 32)
    classes = np.zeros((V, 3), dtype=np.uint32)
    for v in range(V):
        row = list(vv_rows[v])
        if rng is not None and row:
            # plant racy duplicates (later slots repeating an earlier entry)
            for _ in range(int(rng.integers(0, 3))):
                if len(row) < max_vv:
                    row.append(row[int(rng.integers(0, len(row)))])
        padded = row + [-1] * (max_vv - len(row))
        n_index = len(row)
        mask = [True] * max_vv
        valence = [0] * max_vv
        nbh = [None] * max_vv
        my2d = padded
        for t in range(max_vv):
            if my2d[t] < 0 or n_index <= 0:
                mask[t] = False
            if any(padded[i] == my2d[t] for i in range(t)):   # prefix-scan dedup
                mask[t] = False
        for t in range(max_vv):
            if mask[t]:
                u = my2d[t]
                lower = (u < v) if field[u] == field[v] else (field[u] < field[v])
                valence[t] = 1 - (int(lower) << 1)
                nbh[t] = u
        edits = [1, 1]
        it = 0
        while not (edits[0] == 0 and edits[1] == 0) and it < max_vv:
            edits = [0, 0]
            it += 1
            for t in range(max_vv):
                if not mask[t]:
                    continue
                for i in range(n_index):
                    if i != t and valence[i] == valence[t]:
                        cand = padded[i]
                        if my2d[t] in vv_rows[cand] and nbh[t] > nbh[i]:
                            nbh[t] = nbh[i]
                            edits[(valence[t] + 1) // 2] += 1
        for t in range(max_vv):
            if mask[t] and nbh[t] == my2d[t]:
                classes[v, (valence[t] + 1) // 2] += 1
        up, lo = classes[v, 0], classes[v, 1]     # the kernel's own names
        if up >= 1 and lo == 0:
            code = 2
        elif up == 0 and lo >= 1:
            code = 1
        elif up == 1 and lo == 1:
            code = 3
        else:
            code = 4
        classes[v, 2] = code
    return classes


def vv_rows_of(oracle, tvs, n_verts):
    off, ent = oracle.extract(tvs, n_verts, mask=1 << 13)["VV"]
    return [set(ent[off[i]:off[i + 1]].tolist()) for i in range(n_verts)], \
        [ent[off[i]:off[i + 1]].tolist() for i in range(n_verts)]


@pytest.mark.parametrize("seed,frac,dims,quantize", [(1, 0.0, 3, False), (2, 0.5, (3, 2, 3), False),
                                                     (3, 0.3, 3, True)])
def test_oracle_matches_kernel_simulation(oracle, seed, frac, dims, quantize):
    m = meshgen.kuhn_mesh(dims, frac, seed=seed)
    field = meshgen.gaussian_mixture_field(m.coords, n_gauss=5, seed=seed + 10)
    if quantize:  # many exact ties, exercising the id tie-break
        field = (np.round(field * 3) / 3).astype(np.float32)
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    sets, lists = vv_rows_of(oracle, tvs, m.n_verts)
    sim_rows = [sorted(s) for s in sets]
    want = simulate_reference_kernel(sim_rows, field.astype(np.float64),
                                     rng=np.random.default_rng(seed))
    # the simulation tests membership against sets
    got = oracle.critical_points(tvs, m.n_verts, field)
    assert np.array_equal(got, want)


def test_linear_field_known_answer(oracle):
    """A generic linear field on a Kuhn grid: exactly one minimum (code 1) at
    the lowest corner, one maximum (code 2) at the highest, all else regular."""
    m = meshgen.kuhn_mesh(5, 0.0, seed=0, permute=False, shuffle_slots=False)
    x = m.coords.astype(np.float64)
    field = x[:, 0] + 2.1 * x[:, 1] + 4.3 * x[:, 2]
    cp = oracle.critical_points(m.tv, m.n_verts, field)
    assert np.bincount(cp[:, 2], minlength=5).tolist() == [0, 1, 1, m.n_verts - 2, 0]
    assert cp[int(np.argmin(field)), 2] == 1 and cp[int(np.argmax(field)), 2] == 2


def test_single_bump_has_one_maximum(oracle):
    m = meshgen.kuhn_mesh(8, 0.2, seed=4)
    c = np.array([0.52, 0.47, 0.5])
    field = np.exp(-((m.coords.astype(np.float64) - c) ** 2).sum(1) / 0.05)
    cp = oracle.critical_points(oracle.canonicalize(m.tv, m.n_verts), m.n_verts, field)
    assert int((cp[:, 2] == 2).sum()) == 1
    assert cp[int(np.argmax(field)), 2] == 2
