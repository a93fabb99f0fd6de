"""The measured-data readers against the reference's own readers
(Source/sc_readdata.cpp compiled with Qt stand-ins, oracle/build_ref.sh):
image extents, data bit for bit and meta information on the committed
input files of tests/golden/readers/, and the beam-centre finder, from the
fixtures tests/golden/make_readers_golden.py stored; live against the
reference's build where it is present."""
import json
import os

import numpy as np
import pytest

from crystalscatter_gb300 import readers as R
from oracle import refbind

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
with open(os.path.join(GOLD, "readers_ref.json")) as f:
    REF = json.load(f)
ARR = dict(np.load(os.path.join(GOLD, "readers_ref.npz")))
READ = {"kws": R.read_kws, "edf": R.read_edf, "spreadsheet": R.read_spreadsheet,
        "sascrystal": R.read_sascrystal_csv, "tiff": R.read_tiff, "2dsans": R.read_2dsans}


def ours(kind, path):
    try:
        return READ[kind](path)
    except ValueError:
        return None  # the reference's reader returns no image


def _meta(pairs):
    m = {}
    for k, v in pairs:
        m[k] = os.path.basename(v) if k == "From File" else v
    return m


@pytest.mark.parametrize("name", sorted(REF["images"]))
def test_reader_matches_reference(name):
    rec = REF["images"][name]
    img = ours(rec["kind"], os.path.join(GOLD, "readers", rec["file"]))
    if "dims" not in rec:
        assert img is None
        return
    assert img is not None
    assert [img.minX, img.maxX, img.minY, img.maxY] == rec["dims"]
    assert np.array_equal(img.data, ARR[name])
    assert _meta(img.meta.items()) == _meta(rec["meta"])


@pytest.mark.parametrize("name", sorted(REF["beam_center"]))
def test_beam_center_matches_reference(name):
    rec = REF["beam_center"][name]
    x0, x1, y0, y1 = rec["dims"]
    img = R.Image(ARR["beam_" + name], x0, x1, y0, y1)
    assert list(R.find_beam_center(img, *rec["start"])) == rec["center"]


@pytest.mark.skipif(not refbind.readers_available(), reason="the reference's readers are not built here")
@pytest.mark.parametrize("name", sorted(REF["images"]))
def test_fixture_is_the_reference_output(name):
    rec = REF["images"][name]
    r = refbind.read_image(rec["kind"], os.path.join(GOLD, "readers", rec["file"]))
    if "dims" not in rec:
        assert r is None
        return
    assert r["dims"] == rec["dims"] and np.array_equal(r["data"], ARR[name])
    assert _meta(r["meta"]) == _meta(rec["meta"])
