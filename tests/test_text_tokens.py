"""Host checks of the token-parallel reading of long lines of values (no GPU).

The warp-per-line kernels read a line token by token in parallel when every
blank-separated token is, as a whole, one number of the std::istream double
grammar  [sign] (digits [. digits] | . digits) [(e|E) [sign] digits].  For such
a line the extraction loop of SimpleState::readFromFile (the oracle's
getline + istringstream restatement) must return exactly the tokens' values in
order; a token outside the grammar must be one for which a token-wise reading
would be wrong, so that the kernels hand its line to the sequential loop.
"""
import re

import numpy as np
import pytest

import oracle.bind as ob

GRAMMAR = re.compile(rb"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")
BLANKS = [b" ", b"\t", b"  ", b"\v", b"\f", b" \t ", b"\r "]


def _digits(g, lo, hi):
    return "".join(g.choice(list("0123456789"), int(g.integers(lo, hi + 1)))).encode()


def _number(g):
    form = int(g.integers(0, 4))
    if form == 0:
        body = _digits(g, 1, 25)
    elif form == 1:
        body = _digits(g, 1, 12) + b"."
    elif form == 2:
        body = _digits(g, 1, 12) + b"." + _digits(g, 1, 12)
    else:
        body = b"." + _digits(g, 1, 12)
    sign = [b"", b"+", b"-"][int(g.integers(0, 3))]
    exp = b""
    if g.random() < 0.3:
        exp = [b"e", b"E"][int(g.integers(0, 2))] + [b"", b"+", b"-"][int(g.integers(0, 3))] + \
            str(int(g.integers(0, 21))).encode()
    return sign + body + exp


@pytest.mark.parametrize("seed", range(4))
def test_regular_line_reads_as_its_tokens(built, seed):
    g = np.random.default_rng(seed)
    lines, want = [], []
    for _ in range(20):
        toks = [_number(g) for _ in range(int(g.integers(1, 400)))]
        assert all(GRAMMAR.fullmatch(t) for t in toks)
        parts = [BLANKS[int(g.integers(0, len(BLANKS)))]]
        for t in toks:
            parts += [t, BLANKS[int(g.integers(0, len(BLANKS)))]]
        lines.append(b"".join(parts))
        want += [float(t) for t in toks]
    got = ob.parse_values(b"\n".join(lines) + b"\n")
    assert got.shape == (len(want),)
    assert np.array_equal(got, np.array(want))
    assert np.array_equal(np.signbit(got), np.signbit(np.array(want)))


@pytest.mark.parametrize("tok", [b"1.5-2.5", b"1.5.5", b"1e", b"7.5e+", b"abc", b"--1", b"+", b".", b"1e5x",
                                 b"0x10", b"1,5", b"-.e1", b"inf", b"nan", b"1_0"])
def test_irregular_token_defeats_a_token_wise_reading(built, tok):
    assert GRAMMAR.fullmatch(tok) is None
    got = ob.parse_values(b"1 " + tok + b" 2\n")
    try:
        token_wise = [1.0, float(tok), 2.0]
    except ValueError:
        token_wise = None
    assert token_wise is None or not np.array_equal(got, token_wise)


def test_value_count_bound(built):
    """Two extracted values need a non-digit between their digits, so a text
    of n bytes yields at most (n + 1) // 2 values (the output size the
    parse wrapper allocates); dense texts reach it."""
    for text in (b"1-1-1-1-1", b"1 1 1 1\n", b".5.5.5.5", b"1\n2\n3\n", b"1..5", b"7"):
        assert len(ob.parse_values(text)) <= (len(text) + 1) // 2
    assert len(ob.parse_values(b"1-1-1-1-1")) == 5
    g = np.random.default_rng(5)
    alphabet = np.frombuffer(b"0123456789.-+eE \n\t", dtype=np.uint8)
    for _ in range(300):
        text = g.choice(alphabet, int(g.integers(1, 200))).tobytes()
        assert len(ob.parse_values(text)) <= (len(text) + 1) // 2


def test_exact_fast_path_is_correctly_rounded():
    """The device conversion's fast path (Clinger 1990): for a decimal
    mantissa m < 2^53 and exponent |e| <= 22, one IEEE multiplication or
    division of float(m) (exact) by 10^|e| (exact in binary64) gives the
    correctly rounded value of m * 10^e."""
    g = np.random.default_rng(3)
    cases = [(2 ** 53 - 1, 22), (2 ** 53 - 1, -22), (1, -22), (9007199254740991, -1), (1, 0), (0, 5)]
    cases += [(int(g.integers(0, 2 ** 53)), int(g.integers(-22, 23))) for _ in range(20000)]
    cases += [(int(g.integers(0, 10 ** int(g.integers(1, 16)))), int(g.integers(-22, 23))) for _ in range(5000)]
    for m, e in cases:
        p = float(f"1e{abs(e)}")
        v = float(m) * p if e >= 0 else float(m) / p
        assert v == float(f"{m}e{e}"), (m, e)
