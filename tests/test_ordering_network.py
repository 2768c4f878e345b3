"""The candidate ordering of the subnode test (octree_fsh.c:276-290) is a
selection network that swaps two slots when the later one's t is strictly
less. The shader fills the valid bisecting-plane hits into consecutive slots
after the entry point; the CUDA walker instead leaves an invalid hit in its
slot with t = +inf. These tests show, for every validity pattern and every
pattern of equal t values, that both orders keep the valid candidates first
and in the same sequence: the 3-slot network the walker runs when the entry
comes first, and the full 4-slot one."""
import itertools

INF = float("inf")


def _network(slots, first):
    a = list(slots)
    for i in range(first, len(a) - 1):
        for j in range(i + 1, len(a)):
            if a[j][0] < a[i][0]:
                a[i], a[j] = a[j], a[i]
    return a


def _valid(slots):
    return [s for s in slots if s[1] is not None]


def _check(n_hits, with_entry):
    values = [float(v) for v in range(1, n_hits + 2)]
    cases = 0
    for valid in itertools.product((False, True), repeat=n_hits):
        for ts in itertools.product(values, repeat=n_hits + (1 if with_entry else 0)):
            head = [(ts[0], "entry")] if with_entry else []
            hits = [(ts[len(head) + k], "zxy"[k]) for k in range(n_hits)]
            packed = head + [h for h, v in zip(hits, valid) if v]
            packed += [(INF, None)] * (len(head) + n_hits - len(packed))
            in_place = head + [h if v else (INF, None) for h, v in zip(hits, valid)]
            assert _valid(_network(packed, 0)) == _valid(_network(in_place, 0)), (valid, ts)
            cases += 1
    return cases


def test_three_slot_network_in_place_equals_compacted():
    assert _check(3, with_entry=False) == 8 * 4 ** 3


def test_four_slot_network_in_place_equals_compacted():
    assert _check(3, with_entry=True) == 8 * 4 ** 4
