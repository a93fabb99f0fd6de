"""The workload definitions: the sweep's generator is std::mt19937_64 (known
answer of the C++ standard) and the sweep has the stated size distribution."""
from crystalscatter_gb300 import configs as C


def test_mt19937_64_known_answer():
    # [rand.predef]: the 10000th consecutive invocation of a default-constructed
    # std::mt19937_64 produces 9981545732273789042
    r = C.MT19937_64(5489)
    for _ in range(9999):
        r()
    assert r() == 9981545732273789042


def test_sweep_sets_in_stated_ranges():
    sets = C.bct_sweep(4096)
    sizes = {s["EditPixelNoX"] for s in sets}
    assert sizes == {128, 256, 512, 1024}
    for s in sets:
        assert 3 <= s["EditRadius"] < 10 and 20 <= s["Length"] < 100 and 20 <= s["uca"] < 60
        assert 1.0 <= s["ucc"] / s["uca"] < 1.6 and 0.05 <= s["EditSigma"] < 0.20 and 2 <= s["EditAzi"] < 20
        assert s["EditPixelNoX"] == s["EditPixelNoY"] == 2 * s["GridPoints"]
        assert (s["LType"], s["Ordis"], s["ComboBoxParticle"], s["HKLmax"]) == (8, 6, 1, 3)
    total = sum(s["EditPixelNoX"] ** 2 for s in sets)
    assert 1.3e9 < total < 1.5e9
    assert C.bct_set(7) == C.bct_set(7)
