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


def same_spin_double_sign(S: int, i: int, j: int, a: int, b: int) -> int:
    """TwoExcite's rule on one spin's string (spatial orbitals, no spin flip)."""
    I, J, A, B = min(i, j), max(i, j), min(a, b), max(a, b)
    s = parity_between(S, min(I, A), max(I, A)) ^ parity_between(S, min(J, B), max(J, B))
    return s ^ (1 if (A > J or B < I) else 0)


def eta(A: int, B: int, L: int) -> int:
    """Sign (as a parity) between the interleaved determinant and the block one
    (all alpha creators, then all beta): one transposition per (alpha p, beta q)
    pair with q < p."""
    return sum(bin(B & ((1 << p) - 1)).count("1") for p in range(L) if A >> p & 1) & 1


def eta_prefix(A: int, B: int, L: int) -> int:
    """The same parity from the prefix parity of B: bit p of P is the parity of
    the beta bits below p, and eta = parity(P & A)."""
    P, x = 0, 0
    for p in range(L):
        P |= x << p
        x ^= B >> p & 1
    return bin(P & A).count("1") & 1


@pytest.mark.parametrize("L,na,nb", [(5, 2, 2), (6, 3, 2), (6, 2, 3), (7, 3, 3)])
def test_block_order_signs(L, na, nb):
    """Every phase of the reference (interleaved determinant) equals
    eta(bra) + eta(ket) + the phase in the block ordering, which depends on the
    excited spin's own string only: singles and same-spin doubles on their
    string, alpha-beta doubles the product of the two single phases on the bra
    strings.  So a solver whose vectors are multiplied by eta needs no
    opposite-spin parity at all."""
    astrs = [sum(1 << p for p in c) for c in itertools.combinations(range(L), na)]
    bstrs = [sum(1 << p for p in c) for c in itertools.combinations(range(L), nb)]
    occ = lambda s: [p for p in range(L) if s >> p & 1]
    vir = lambda s: [p for p in range(L) if not s >> p & 1]
    checked = 0
    for A in astrs:
        for B in bstrs:
            det = interleave(A, B, L)
            e0 = eta(A, B, L)
            assert e0 == eta_prefix(A, B, L)
            for i in occ(A):  # alpha singles
                for a in vir(A):
                    A2 = A ^ (1 << i) ^ (1 << a)
                    assert one_excite_sign(det, 2 * i, 2 * a) == e0 ^ eta(A2, B, L) ^ parity_between(A, min(i, a), max(i, a))
                    for j in occ(B):  # alpha x beta
                        for b in vir(B):
                            B2 = B ^ (1 << j) ^ (1 << b)
                            ref = two_excite_sign(det, 2 * i, 2 * j + 1, 2 * a, 2 * b + 1)
                            blk = parity_between(A, min(i, a), max(i, a)) ^ parity_between(B, min(j, b), max(j, b))
                            assert ref == e0 ^ eta(A2, B2, L) ^ blk
                            checked += 1
            for j in occ(B):  # beta singles
                for b in vir(B):
                    B2 = B ^ (1 << j) ^ (1 << b)
                    assert one_excite_sign(det, 2 * j + 1, 2 * b + 1) == e0 ^ eta(A, B2, L) ^ parity_between(B, min(j, b), max(j, b))
            for S, spin in ((A, 0), (B, 1)):  # same-spin doubles
                o, v = occ(S), vir(S)
                for i, j in itertools.combinations(o, 2):
                    for a, b in itertools.combinations(v, 2):
                        S2 = S ^ (1 << i) ^ (1 << j) ^ (1 << a) ^ (1 << b)
                        ref = two_excite_sign(det, 2 * i + spin, 2 * j + spin, 2 * a + spin, 2 * b + spin)
                        ket = eta(S2, B, L) if spin == 0 else eta(A, S2, L)
                        assert ref == e0 ^ ket ^ same_spin_double_sign(S, i, j, a, b)
                        checked += 1
    assert checked > 0
