"""TSPLIB reader (aco_tsplib_*): the parsing rules of the reference's
TSPReader::read on written files, its error cases, and -- where the reference
tree is present -- every instance it ships, with the published optima as a
lower bound on tours built from the parsed coordinates."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

import oracle
from acogpu_gb300 import _abi, instances
from acogpu_gb300.colony import AcoError
from acogpu_gb300 import tsplib

REF = oracle.REF_SOURCES
INPUT = os.path.join(REF, "release", "input")
_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]


def strtof(tok):
    """The float sscanf("%f") stores for a decimal token."""
    return np.float32(_libc.strtof(tok.encode(), None))


def independent_parse(path):
    """A second reading of a well-formed EUC_2D file: tokens after
    NODE_COORD_SECTION, DIMENSION lines, coordinates through strtof."""
    lines = open(path, newline="").read().replace("\r", "").split("\n")
    n, name, xs, ys = None, None, [], []
    it = iter(lines)
    for line in it:
        key = line.split(":")[0].replace(" ", "")
        if key == "NAME":
            name = line.split(":", 1)[1].replace(" ", "")
        elif key == "DIMENSION":
            n = int(line.split(":", 1)[1])
        elif key == "NODE_COORD_SECTION":
            for _ in range(n):
                tok = next(it).split()
                xs.append(strtof(tok[1]))
                ys.append(strtof(tok[2]))
            break
    return name, np.array(xs, np.float32), np.array(ys, np.float32)


def write(path, text, crlf=False):
    data = text.replace("\n", "\r\n") if crlf else text
    with open(path, "w", newline="") as f:
        f.write(data)
    return str(path)


GOOD = """NAME : tiny7
COMMENT : written by the test (spaces, a CR, a comment)
TYPE : TSP
DIMENSION : 7
EDGE_WEIGHT_TYPE : EUC_2D
NODE_COORD_SECTION
1 0 0
2 3.5 4.25
3 1e2 7
4 0.1 0.2
5 100000 99999.5
6 -3 2
7 12345.678 0.333333333
EOF
"""


@pytest.mark.parametrize("crlf", [False, True])
def test_reads_fields_and_coordinates(tmp_path, crlf):
    inst = tsplib.read(write(tmp_path / "tiny7.tsp", GOOD, crlf))
    assert inst.name == "tiny7" and inst.n == 7
    toks = [l.split() for l in GOOD.splitlines()[6:13]]
    assert np.array_equal(inst.x, np.array([strtof(t[1]) for t in toks], np.float32))
    assert np.array_equal(inst.y, np.array([strtof(t[2]) for t in toks], np.float32))


def test_stsp_type_and_missing_eof_are_accepted(tmp_path):
    text = GOOD.replace("TYPE : TSP", "TYPE: STSP").replace("EOF\n", "")
    assert tsplib.read(write(tmp_path / "a.tsp", text)).n == 7


@pytest.mark.parametrize("edit,status", [
    (("TYPE : TSP", "TYPE : ATSP"), _abi.ACO_ERR_FORMAT),
    (("EUC_2D", "GEO"), _abi.ACO_ERR_FORMAT),
    (("DIMENSION : 7", "DIMENSION : 9"), _abi.ACO_ERR_FORMAT),      # EOF inside the section
    (("DIMENSION : 7\n", ""), _abi.ACO_ERR_FORMAT),                # section before a size
    (("4 0.1 0.2", "4 0.1"), _abi.ACO_ERR_FORMAT),                 # short coordinate line
])
def test_rejected_files(tmp_path, edit, status):
    text = GOOD.replace(*edit)
    with pytest.raises(AcoError) as e:
        tsplib.read(write(tmp_path / "bad.tsp", text))
    assert e.value.status == status


def test_missing_file(tmp_path):
    with pytest.raises(AcoError) as e:
        tsplib.read(tmp_path / "none.tsp")
    assert e.value.status == _abi.ACO_ERR_IO


def test_generated_instance_round_trip(tmp_path):
    """An instance of the synthetic generator written in TSPLIB form reads back
    bit for bit (integer coordinates are exact in float)."""
    x, y = instances.clustered_instance(300, seed=5)
    body = "".join(f"{i + 1} {int(a)} {int(b)}\n" for i, (a, b) in enumerate(zip(x, y)))
    text = f"NAME: gen300\nTYPE: TSP\nDIMENSION: 300\nEDGE_WEIGHT_TYPE: EUC_2D\n" \
           f"NODE_COORD_SECTION\n{body}EOF\n"
    inst = tsplib.read(write(tmp_path / "gen300.tsp", text))
    assert np.array_equal(inst.x, x.astype(np.float32))
    assert np.array_equal(inst.y, y.astype(np.float32))
    assert np.array_equal(oracle.distances(inst.x, inst.y), instances.euc2d_distances(x, y))


def _reference_files():
    if not os.path.isdir(INPUT):
        return []
    return sorted(f for f in os.listdir(INPUT) if f.endswith(".tsp"))


def _optima():
    out = {}
    path = os.path.join(INPUT, "tsplip-opt.txt")
    for line in open(path):
        if ":" in line:
            k, v = line.split(":")
            out[k.strip()] = int(v)
    return out


@pytest.mark.skipif(not _reference_files(), reason="reference inputs absent")
@pytest.mark.parametrize("fname", _reference_files() or ["none"])
def test_reference_instances_parse(fname):
    path = os.path.join(INPUT, fname)
    inst = tsplib.read(path)
    name, x, y = independent_parse(path)
    assert inst.name == name == fname[:-4]
    assert np.array_equal(inst.x, x) and np.array_equal(inst.y, y)


@pytest.mark.skipif(not _reference_files(), reason="reference inputs absent")
@pytest.mark.parametrize("name", ["berlin52", "eil76", "kroA100"])
def test_tours_on_reference_instances_respect_the_optimum(name):
    """Distances of the parsed coordinates (the reference's EUC_2D rule):
    tours built by the oracle are never shorter than the published optimum,
    and after a few iterations come within 15% of it."""
    inst = tsplib.read(os.path.join(INPUT, name + ".tsp"))
    d = oracle.distances(inst.x, inst.y)
    opt = _optima()[name]
    p = _abi.default_params(num_ants=inst.n, beta=2.0, rho=0.5, cand_k=20,
                            nn_order=_abi.ACO_NN_STABLE, fallback=_abi.ACO_FALLBACK_BEST,
                            tau0_mode=_abi.ACO_TAU0_DORIGO, seed=3)
    q = oracle.Port(p, d, threads=4)
    q.initialize()
    q.iterate(30)
    assert q.glob_best() >= opt
    assert q.glob_best() <= 1.15 * opt
    assert np.all(q.lengths() >= opt)
    q.close()
