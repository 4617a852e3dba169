"""iqs_gb300.Permutation and GateCounter (host logic) against the reference's own unit tests
(unit_test/include/permutation_test.hpp:46-257, gate_counter_test.hpp)."""
import pytest


def test_identity_and_basic_use():
    from iqs_gb300 import Permutation
    p = Permutation(6)
    assert p.num_elements == 6 and [p[i] for i in range(6)] == list(range(6))
    m, im = [1, 2, 0, 3, 5, 4], [2, 0, 1, 3, 5, 4]
    p.SetNewPermutationFromMap(m, "direct")
    assert p.map == m and p.imap == im
    p.SetNewPermutationFromMap(m, "inverse")
    assert p.imap == m and p.map == im


def test_exchange_two_elements():
    from iqs_gb300 import Permutation
    p = Permutation([1, 2, 0, 3, 5, 4])
    m = [1, 2, 0, 3, 5, 4]
    for e1, e2 in ((2, 4), (4, 0)):
        m[e1], m[e2] = m[e2], m[e1]
        p.ExchangeTwoElements(e1, e2)
        assert p.map == m and all(p.imap[m[i]] == i for i in range(6))


def test_program2data_and_data2program():
    from iqs_gb300 import Permutation
    p = Permutation(3)
    assert [p.program2data_(v) for v in range(8)] == list(range(8))
    p.SetNewPermutationFromMap([1, 0, 2])
    assert [p.program2data_(v) for v in range(8)] == [0, 2, 1, 3, 4, 6, 5, 7]
    assert all(p.data2program_(v) == p.program2data_(v) for v in range(8))
    p.SetNewPermutationFromMap([1, 2, 0])
    assert [p.program2data_(v) for v in range(8)] == [0, 2, 4, 6, 1, 3, 5, 7]
    q = Permutation(4)
    q.SetNewPermutationFromMap([2, 3, 1, 0], "inverse")
    want = [0, 4, 8, 12, 2, 6, 10, 14, 1, 5, 9, 13, 3, 7, 11, 15]
    assert [q.data2program_(v) for v in range(16)] == want
    assert [q.bin2dec(q.data2program(v)) for v in range(16)] == want
    assert all(q.program2data(q.data2program(v)) == q.dec2bin(v, 4) for v in range(16))


def test_intermediate_inverse_maps():
    from iqs_gb300 import Permutation
    p = Permutation(list(range(8)))
    assert p.ObtainIntemediateInverseMaps([1, 5, 2, 3, 6, 0, 7, 4], 5) == ([1, 0, 2, 3, 4, 5, 6, 7],
                                                                          [1, 0, 2, 3, 4, 5, 7, 6])
    p.SetNewPermutationFromMap([1, 5, 2, 3, 6, 0, 7, 4])
    assert p.ObtainIntemediateInverseMaps([1, 6, 7, 4, 3, 2, 0, 5], 5) == ([2, 0, 5, 7, 3, 1, 4, 6],
                                                                          [2, 0, 5, 7, 3, 4, 1, 6])


def test_strings_find_and_errors(capsys):
    from iqs_gb300 import Permutation
    p = Permutation([2, 0, 1])
    assert p.Find(0) == 1 and p.GetMapStr() == " 2 0 1" and p.GetImapStr() == " 1 2 0"
    assert p.Print() == "qubit permutation:  2 0 1"
    assert capsys.readouterr().out == "qubit permutation:  2 0 1\n"
    with pytest.raises(ValueError):
        p.SetNewPermutationFromMap([0, 0, 1])


def test_gate_counter():
    from iqs_gb300 import GateCounter
    g = GateCounter(4)
    g.OneQubitIncrement(0)
    g.OneQubitIncrement(0)
    g.TwoQubitIncrement(0, 3)
    g.OneQubitIncrement(2)
    assert (g.GetOneQubitGateCount(), g.GetTwoQubitGateCount(), g.GetTotalGateCount()) == (3, 1, 4)
    assert g.GetParallelDepth() == 3
