"""Input edge cases of the problem parser (host only, no GPU).

The library's parser follows src/problem.cc:183-247: the header, the index
base chosen by the file name, a missing weight meaning 1, blank lines
skipped, the dense/sparse choice at 10 % density (duplicate lines are
parallel edges in sparse files and overwrite in dense ones).  Each case, and
each text-layout variant (CRLF, tabs, trailing blanks, no final newline, a
header counting more edges than follow), is compared with the oracle's parse
of the same file.  Inputs the engine cannot
represent exactly are refused with a status code; the product has no CPU
path, so creating a context without a GPU fails loudly.
"""
import math
import os

import pytest

from oracle import pyoracle as O

CASES = {
    "isolated": "5 0\n",
    "single": "1 0\n",
    "noweights": "4 3\n1 2\n2 3\n3 4\n",
    "zero.gset": "3 2\n0 1 1\n1 2 -1\n",
    "dup_dense": "3 2\n1 2 1\n1 2 1\n",
    "dup_sparse": "50 3\n1 2 1\n1 2 1\n3 4 -1\n",
    "blankline": "3 1\n1 2 1\n\n",
    "lin.ising": "3 2 1\n0 1\n2 -1\n0 1 2\n",
}

# text-layout variants, parsed on the host only
LAYOUT_CASES = {
    "short_header": "3 5\n1 2 1\n2 3 -1\n",        # fewer lines than the header's M (M still scales)
    "crlf": "3 2\r\n1 2 1\r\n2 3 -1\r\n",
    "tabs": "3 2\n1\t2\t1\n2\t3\t-1\n",
    "trailing_space": "3 2\n1 2 1 \n2 3 -1   \n",
    "blank_end": "3 2\n1 2 1\n2 3 -1\n\n\n",
    "no_final_newline": "3 2\n1 2 1\n2 3 -1",
    "plus_sign": "3 2\n1 2 +1\n2 3 -1\n",
    "float_int": "3 2\n1 2 1.0\n2 3 -2.0\n",
}

REJECTED = {
    "selfloop": ("2 1\n1 1 1\n", 3),
    "fraction": ("2 1\n1 2 0.5\n", 3),
    "too_big": ("2 1\n1 2 200\n", 3),
    "empty": ("", 2),
    "out_of_range": ("2 1\n1 3 1\n", 2),
}


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode())   # line endings as given
    return str(p)


@pytest.mark.parametrize("name", sorted(CASES) + sorted(LAYOUT_CASES))
def test_parse_matches_oracle(tmp_path, name):
    import pticm
    path = _write(tmp_path, name, CASES.get(name) or LAYOUT_CASES[name])
    info = pticm.Problem.load(path).info()
    orc = O.Problem.load(path, 0)
    assert info.n == orc.n and info.m == orc.m
    assert bool(info.sparse) == orc.sparse
    if math.isnan(orc.char_scale):
        assert math.isnan(info.char_scale)
    else:
        assert info.char_scale == orc.char_scale
    row, col, w = orc.adjacency()
    # directed entries: parallel edges stay separate in sparse files, a
    # repeated pair is one entry per direction in dense ones
    assert info.nnz == (len(col) if orc.sparse else int((w != 0).sum()))
    assert info.ncolors >= 1


@pytest.mark.parametrize("name", sorted(REJECTED))
def test_unrepresentable_inputs_are_refused(tmp_path, name):
    import pticm
    text, code = REJECTED[name]
    path = _write(tmp_path, name, text)
    with pytest.raises(pticm.PticmError) as e:
        pticm.Problem.load(path)
    assert e.value.code == code


def test_context_without_a_gpu_fails_loudly():
    import pticm
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    prob = pticm.Problem.load(os.path.join(os.path.dirname(__file__), "golden", "graphs", "pmL6.gset"))
    with pytest.raises(pticm.PticmError) as e:
        pticm.Context(prob, nt=4, seed=1)
    assert e.value.code == 7   # PTICM_ERR_NODEVICE: the engine has no CPU path
