"""Parameter keys, combobox texts and the console key/value string."""
import crystalscatter_gb300 as cs


def fresh():
    return cs.SasCalc_GENERIC_calculation()


def test_reference_keys_set_fields():
    c = fresh()
    c.setParams({"EditRadius": 7.5, "ComboBoxParticle": 1, "Ordis": 6, "LType": 8, "HKLmax": 3,
                 "EditPixelX": 0.172, "CenterBeam": 1, "RadioButtonQ1": 1, "ExpandImage": 1, "Editdom2": 12})
    p = c.params()
    assert (p.radius, p.particle, p.ordis, p.ltype, p.hklmax) == (7.5, 1, 6, 8, 3)
    assert p.pixx_mm == 0.172 and p.usebeamstop == 1 and p.radq1 == 1 and p.expand == 1
    assert p.sigxyz[1] == 12


def test_unknown_key_rejected():
    c = fresh()
    try:
        c.setParam("NoSuchKey", 1.0)
        ok = False
    except cs.CrystalScatterError as e:
        ok = e.code == cs.CS_ERR_PARAM
    assert ok


def test_combobox_text():
    c = fresh()
    c.setParam("ComboBoxParticle", "cylinder")
    c.setParam("Ordis", "z-dir")
    c.setParam("ComboBoxInterior", "core + homogeneous sh")
    c.setParam("ComboBoxPeak", "Pearson VII")
    c.setParam("LType", "BCT (l4/mm)")
    p = c.params()
    assert (p.particle, p.ordis, p.interior, p.peak, p.ltype) == (1, 6, 1, 5, 8)
    c.setParam("ComboBoxParticle", "Sphere")  # case-sensitive: not in the list
    assert c.params().particle == -1


def test_mcpval_string_rules():
    c = fresh()
    c.setKeyValues("radius=12.5;cbparticle=cylinder;ordis=Gaussian;sigma=0.2;debyescherrer=T;"
                   "rbpara=False;i0=2;unknown=3;gridpoints=64;qmax=NULL;length=;pixelx=.5")
    p = c.params()
    assert p.radius == 12.5 and p.particle == 1 and p.ordis == 0 and p.sigma == 0.2
    assert p.debyescherrer == 1 and p.para == 0 and p.izero == 2 and p.gridpoints == 64
    assert p.qmax == 1 and p.length == 1  # NULL and empty values leave the parameter unchanged
    assert p.pixx_mm == 1  # ".5" is neither a number nor a combobox text for the console


def test_mcpval_combobox_starting_with_F_is_a_boolean():
    # "FCC (Fm3m)" starts with 'F' and the console reads it as boolean false
    c = fresh()
    c.setKeyValues("ltype=FCC (Fm3m)")
    assert c.params().ltype == 0
    c.setKeyValues("ltype=5")
    assert c.params().ltype == 5


def test_mcpval_hidden_keys_ignored():
    c = fresh()
    c.setKeyValues("centerbeam=T;expandimage=T;editqmin=3;p1=4")
    p = c.params()
    assert p.usebeamstop == 0 and p.expand == 0 and p.qmin == 0 and p.p1 == 0
