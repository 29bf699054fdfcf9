"""The alpha-beta phase factorises into single-excitation phases.

The reference evaluates an alpha-single x beta-single element with TwoExcite
on the bra determinant (chemistry/basic/determinants.h:500-518; parity rule
:242-294, spin orbitals interleaved alpha 2p / beta 2p+1, :105-150), taking
the minus sign of the exchange-type integral when A and I have different
spins.  The sigma kernel instead multiplies the alpha single's phase on the
bra by the beta single's phase on the determinant after the alpha move.  This
test checks that identity exhaustively for every string pair and every
alpha/beta single excitation on small orbital sets.
"""
import itertools

import pytest


def parity_between(det: int, s: int, e: int) -> int:
    """Reference parity(det, s, e): bits in [s, e), flipped again when bit s is set
    (determinants.h:242-294) -- i.e. the bits strictly between s and e."""
    cnt = bin(det & (((1 << e) - 1) ^ ((1 << s) - 1))).count("1")
    if det >> s & 1:
        cnt += 1
    return cnt & 1


def interleave(a: int, b: int, L: int) -> int:
    d = 0
    for p in range(L):
        d |= (a >> p & 1) << (2 * p)
        d |= (b >> p & 1) << (2 * p + 1)
    return d


def two_excite_sign(det: int, i: int, j: int, a: int, b: int) -> int:
    I, J, A, B = min(i, j), max(i, j), min(a, b), max(a, b)
    s = parity_between(det, min(I, A), max(I, A)) ^ parity_between(det, min(J, B), max(J, B))
    if A > J or B < I:
        s ^= 1
    # Value(A,I,B,J) vanishes when A, I differ in spin; -Value(A,J,B,I) survives
    if (A & 1) != (I & 1):
        s ^= 1
    return s


def one_excite_sign(det: int, i: int, a: int) -> int:
    return parity_between(det, min(i, a), max(i, a))


@pytest.mark.parametrize("L,na,nb", [(5, 2, 2), (6, 3, 2), (6, 2, 3), (7, 3, 3)])
def test_alpha_beta_sign_is_product_of_single_phases(L, na, nb):
    astrs = [sum(1 << p for p in c) for c in itertools.combinations(range(L), na)]
    bstrs = [sum(1 << p for p in c) for c in itertools.combinations(range(L), nb)]
    checked = 0
    for A in astrs:
        for B in bstrs:
            det = interleave(A, B, L)
            for cra in (p for p in range(L) if A >> p & 1):
                for ana in (p for p in range(L) if not A >> p & 1):
                    Aket = (A & ~(1 << cra)) | (1 << ana)
                    sa = one_excite_sign(det, 2 * cra, 2 * ana)
                    det_after = interleave(Aket, B, L)
                    for crb in (p for p in range(L) if B >> p & 1):
                        for anb in (p for p in range(L) if not B >> p & 1):
                            ref = two_excite_sign(det, 2 * cra, 2 * crb + 1, 2 * ana, 2 * anb + 1)
                            sb = one_excite_sign(det_after, 2 * crb + 1, 2 * anb + 1)
                            assert ref == sa ^ sb, (A, B, cra, ana, crb, anb)
                            checked += 1
    assert checked > 0
