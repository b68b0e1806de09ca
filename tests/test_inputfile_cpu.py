"""The input-file reader (ffe/inputfile.py) against the rules of
src/io/read_input.F90:56-102 (parseInput) and :138-384 (getInput), on input
files written in the reference's `<block>` / `key = value # comment` format
(tests/inputs/)."""
import os

import pytest

import ffe
from conftest import ROOT
from ffe.inputfile import InputError, read_input

INPUTS = os.path.join(ROOT, "tests", "inputs")


def test_pulsar_input_builds_the_descriptor():
    desc, st = ffe.desc_from_input(os.path.join(INPUTS, "input.psr_small"), setup="psr")
    assert (desc.sx, desc.sy, desc.sz) == (96, 96, 96)
    assert (desc.gsx, desc.gsy, desc.gsz) == (96, 96, 96)
    # one absorbing axis makes all three absorbing (src/logistics/initialize.F90:144-148)
    assert list(desc.boundary) == [2, 2, 2] and desc.absorb_buff == 12
    assert abs(desc.cc - 0.45) < 1e-15
    assert desc.setup == ffe.SETUP_PSR
    assert list(desc.params[:4]) == [9.6, 30.0, 402.12386, 1.0]  # psr_bscale defaults to 1
    assert st == {"last": 500, "output_start": 0, "output_interval": 50, "output_istep": 2}


def test_periodic_input_and_the_parser_rules():
    path = os.path.join(INPUTS, "input.periodic_small")
    desc, st = ffe.desc_from_input(path)
    # only the first <grid> block is searched; tabs and blank lines are skipped
    assert (desc.sx, desc.sy, desc.sz) == (32, 24, 16)
    assert list(desc.boundary) == [1, 1, 1]
    assert desc.absorb_buff == 20                    # reference default, unused when periodic
    assert abs(desc.cc - 0.45) < 1e-15               # '4.5d-1'
    assert st["last"] == 200 and st["output_interval"] == 10  # <output> absent: defaults
    f = read_input(path)
    assert f.get("problem", "beta_twist") == 0.25    # the value stops at '#'
    assert f.get("problem", "mx0", int) == 111       # keys are per block
    # 'L0=7.0' is one list-directed token, not the key L0: not found
    assert f.raw("problem", "L0") is None
    assert f.get("problem", "L0", float, 3.0) == 3.0
    with pytest.raises(InputError):
        f.get("problem", "r_L0")                     # no default: an error (read_input.F90:148-156)
    with pytest.raises(InputError):
        ffe.desc_from_input(path, setup="uniform")   # user_uniform needs r_L0, t0 with no default


def test_missing_file_is_an_error():
    with pytest.raises(InputError):
        read_input(os.path.join(INPUTS, "no_such_input"))
