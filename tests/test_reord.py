"""Node reordering (reord, Reord.f:1-44): the library's reverse Cuthill-McKee
(pm_reord, host code) against the oracle's line-by-line restatement of
genrcm_v1 / fnroot_v1 / rcm_v1 / rootls_v1 / degree_v1, bit for bit, and the
deck reader's config block.  CPU only."""
import os

import numpy as np
import pytest

import oracle
import poromec_gb300 as pg
from poromec_gb300 import meshgen

from conftest import load_golden


def _ix(chain):
    """Two-node 'elements' along a chain of node ids (ix rows: a, b, material)."""
    return np.array([[a, b, 1] for a, b in zip(chain[:-1], chain[1:])], np.int32)


def test_rcm_of_a_path_by_hand():
    """A path 3-1-4-5-2: fnroot moves the root from node 1 to the end node 2
    (5 levels against 4), Cuthill-McKee from 2 visits 2 5 4 1 3, reversed."""
    ix = _ix([3, 1, 4, 5, 2])
    expect = [3, 1, 4, 5, 2]
    assert list(pg.reord(5, len(ix), 2, ix)) == expect
    assert list(oracle.reord(5, len(ix), 2, ix)) == expect


def test_rcm_components_and_isolated_nodes():
    """Components are numbered in the order of their lowest node; a node in
    no element is a component of its own."""
    ix = np.concatenate([_ix([6, 2, 7]), _ix([1, 5, 3])])
    a = pg.reord(8, len(ix), 2, ix)
    b = oracle.reord(8, len(ix), 2, ix)
    assert np.array_equal(a, b)
    assert sorted(a) == list(range(1, 9))
    # node 1's component {1, 5, 3} first, then {2, 6, 7}, then the lone 4 and 8
    assert set(a[:3]) == {1, 3, 5} and set(a[3:6]) == {2, 6, 7} and list(a[6:]) == [4, 8]


def _problems():
    out = [meshgen.cube_problem(4), meshgen.tetra_problem(5), meshgen.column_problem(),
           meshgen.union_problem(meshgen.batch_instances(ninst=4, nmin=2, nmax=4, seed=3))]
    for name in ("solo_cilindro_tetra_1", "solo1_tetra", "exemplo1_mesh0_t2"):
        out.append(load_golden(name))
    return out


@pytest.mark.parametrize("k", range(7))
def test_rcm_library_matches_oracle(k):
    pb = _problems()[k]
    a = pg.reord(pb["nnode"], pb["numel"], pb["nen"], pb["ix"])
    b = oracle.reord(pb["nnode"], pb["numel"], pb["nen"], pb["ix"])
    assert np.array_equal(a, b)
    assert np.array_equal(np.sort(a), np.arange(1, int(pb["nnode"]) + 1))


def _bandwidth(pb, num):
    """Largest equation-number distance between two nodes of one element."""
    pos = np.empty(int(pb["nnode"]) + 1, np.int64)
    pos[num] = np.arange(len(num))
    e = pos[pb["ix"][:, :int(pb["nen"])]]
    return int((e.max(1) - e.min(1)).max())


def test_rcm_narrows_a_scrambled_mesh():
    """Node ids of a 10^3 hexa20 cube shuffled: RCM brings the element
    bandwidth (4,942 shuffled) down by more than a factor 3 (to 1,183: the
    width of two of its diagonal level sets)."""
    pb = meshgen.cube_problem(10)
    rng = np.random.default_rng(1)
    perm = rng.permutation(int(pb["nnode"])) + 1
    ix = pb["ix"].copy()
    ix[:, :20] = perm[ix[:, :20] - 1]
    scr = dict(pb, ix=ix)
    nat = np.arange(1, int(pb["nnode"]) + 1)
    num = pg.reord(pb["nnode"], pb["numel"], 20, ix)
    assert _bandwidth(scr, num) * 3 < _bandwidth(scr, nat)


def test_oracle_with_rcm_keeps_the_golden_counts(golden):
    """The tetra cylinder was run with reord true: its neq and nad (an
    ordering invariant) are reproduced with the RCM order, and the order
    changes the pattern (ja) against the natural one."""
    fx = golden("solo_cilindro_tetra_1")
    assert int(fx["reord"]) == 1
    num = oracle.reord(fx["nnode"], fx["numel"], fx["nen"], fx["ix"])
    kw = [int(fx["nnode"]), int(fx["nnodev"]), int(fx["numel"]), int(fx["nen"]),
          int(fx["nenv"]), fx["ix"], fx["id"], fx["fnno"], fx["x"], fx["ie"], fx["e"]]
    o = oracle.Oracle(*kw, num=num)
    assert o.neq == int(fx["neq_ref"]) and o.nad == int(fx["nad_ref"])
    ia, ja, _, _ = o.get_csrd()
    ia0, ja0, _, _ = oracle.Oracle(*kw).get_csrd()
    assert not np.array_equal(ja, ja0)


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)


def test_deck_config_reord(tmp_path):
    """reord defaults to true (reordf, Main.f:255); a config block, inline as
    in the older decks or in a named file, can turn it off."""
    from poromec_gb300 import deck
    from deck_writer import write_linear_deck
    fx = load_golden("exemplo1_mesh0_t2")
    path = write_linear_deck(fx, str(tmp_path), "col", nsteps=1)
    d = deck.Deck(path)
    assert d.value("reord") == 0  # the writer's config block says false
    text = open(path).read()
    assert "reord false" in text
    _write(path, text.replace("reord false", "reord .true."))
    assert deck.Deck(path).value("reord") == 1
    lines = text.split("\n")
    k = lines.index("config")
    assert lines[k + 2] == "end config"
    _write(os.path.join(str(tmp_path), "cfg.dat"), "memory 10\nreord F\nend\n")
    _write(path, "\n".join(lines[:k] + ["config cfg.dat"] + lines[k + 3:]))
    assert deck.Deck(path).value("reord") == 0
    _write(path, "\n".join(lines[:k] + lines[k + 3:]))
    assert deck.Deck(path).value("reord") == 1
