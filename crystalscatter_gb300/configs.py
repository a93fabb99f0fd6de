"""Benchmark and test workloads, as parameter dictionaries keyed by the
reference's own parameter keys (Source/sc_calc_generic.cpp:142-238).

The five workloads restate the synthetic inputs of the benchmark definition:

* ``sphere``        spheres, no lattice, isotropic (pSph_lNon_oIso), 256x256
* ``cyl_gauss``     cylinders, no lattice, Gaussian orientation (pCyl_lNon_oGau),
                    axis in the detector plane at azimuth 30 deg, 512x512. With
                    phi != 0 and theta = 90 the reference's 0-based orientation
                    case reaches no branch of its orientation integrand and the
                    image is 0 beyond 0.4*limq1; this is reproduced.
* ``cyl_gauss_x``   the same with phi = 0 (cylinder axis along x), which runs the
                    full nested Romberg orientation average (labelled supplement)
* ``sphere_fcc``    spheres on FCC, Gaussian peaks and orientation, 1024x1024
* ``cyl_bct``       cylinders on BCT, z-direction orientation; 4096 seeded
                    parameter sets of detector size 128..1024 (``bct_sweep``)

Values that the benchmark text leaves open are fixed here and stated: HKLmax 5
for FCC and 3 for BCT, Debye-Scherrer peak width on, beam centre at the image
centre (CenterBeam with BeamPos 0,0), all four quadrants, no image expansion.
"""

BASE = dict(
    ComboBoxInterior=0, I0=1.0, Base=0.0, iso=0.0, ifluc=0.0, rfluc=0.0,
    CenterBeam=1, BeamPosX=0.0, BeamPosY=0.0, RadioButtonQ1=0, RadioButtonQ2=0, RadioButtonQ4=1, ExpandImage=0,
)

SPHERE = dict(BASE, ComboBoxParticle=0, LType=12, Ordis=7, EditRadius=10.0, EditSigma=0.10,
              GridPoints=128, EditPixelNoX=256, EditPixelNoY=256, EditPixelX=0.5, EditPixelY=0.5,
              EditDet=2.0, EditWavelength=0.6)

CYL_GAUSS = dict(BASE, ComboBoxParticle=1, LType=12, Ordis=0, EditRadius=5.0, EditSigma=0.10, Length=60.0,
                 SigmaL=0.10, theta=90.0, phi=30.0, EditDbeta=15.0,
                 GridPoints=256, EditPixelNoX=512, EditPixelNoY=512, EditPixelX=0.5, EditPixelY=0.5,
                 EditDet=4.0, EditWavelength=0.6)

CYL_GAUSS_X = dict(CYL_GAUSS, phi=0.0)

SPHERE_FCC = dict(BASE, ComboBoxParticle=0, LType=5, ComboBoxPeak=1, Ordis=0, EditRadius=8.0, EditSigma=0.08,
                  uca=40.0, ucb=40.0, ucc=40.0, ucalpha=90.0, ucbeta=90.0, ucgamma=90.0, ucn1=0.0, ucn2=0.0,
                  ucn3=1.0, EditDebyeWaller=1.5, EditDomainSize=300.0, RadButDebyeScherrer=1, EditAzi=5.0,
                  EditDbeta=5.0, HKLmax=5,
                  GridPoints=512, EditPixelNoX=1024, EditPixelNoY=1024, EditPixelX=0.172, EditPixelY=0.172,
                  EditDet=3.0, EditWavelength=0.154)

CYL_BCT_FIXED = dict(BASE, ComboBoxParticle=1, LType=8, ComboBoxPeak=1, Ordis=6, HKLmax=3,
                     RadButDebyeScherrer=1, EditDomainSize=300.0, EditWavelength=0.154, EditDet=3.0,
                     EditPixelX=0.172, EditPixelY=0.172, ucalpha=90.0, ucbeta=90.0, ucgamma=90.0)

WORKLOADS = {
    "sphere": SPHERE,
    "cyl_gauss": CYL_GAUSS,
    "cyl_gauss_x": CYL_GAUSS_X,
    "sphere_fcc": SPHERE_FCC,
}


def scaled(cfg, gridpoints):
    """The same detector q-range on a coarser grid: the pixel size grows by the
    factor the pixel count shrinks (test sizes of the full workloads)."""
    c = dict(cfg)
    s = gridpoints / cfg["GridPoints"]
    c["GridPoints"] = gridpoints
    c["EditPixelNoX"] = 2 * gridpoints
    c["EditPixelNoY"] = 2 * gridpoints
    c["EditPixelX"] = cfg["EditPixelX"] / s
    c["EditPixelY"] = cfg["EditPixelY"] / s
    return c


class MT19937_64:
    """The 64-bit Mersenne Twister (std::mt19937_64: Matsumoto & Nishimura's
    MT19937-64 parameters), so the sweep's parameter sets follow from the
    stated seeds exactly as a C++ std::mt19937_64 would draw them."""

    N, M = 312, 156
    A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed=5489):
        mt = [0] * self.N
        mt[0] = seed & self.MASK
        for i in range(1, self.N):
            mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & self.MASK
        self.mt, self.i = mt, self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.i = 0

    def __call__(self):
        if self.i >= self.N:
            self._twist()
        y = self.mt[self.i]
        self.i += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & self.MASK

    def uniform(self, a, b):
        """a + (b-a) u with u = the top 53 bits of one draw times 2^-53, in [0, 1)."""
        return a + (b - a) * ((self() >> 11) * (1.0 / 9007199254740992.0))

    def choice4(self, seq):
        """one of four items from the top two bits of one draw"""
        return seq[self() >> 62]


def bct_set(k, sizes=(128, 256, 512, 1024)):
    """Parameter set k of the cylinder/BCT sweep: std::mt19937_64 seeded with
    0xC5A70000+k draws, in this order, the detector size N (uniform over
    128/256/512/1024), radius U[3,10] nm, length U[20,100] nm, a U[20,60] nm,
    c/a U[1.0,1.6], the Schulz sigma of radius and length U[0.05,0.20] and the
    orientation width U[2,20] deg. Pixel 0.172 mm, 3 m, 0.154 nm, HKLmax 3."""
    rng = MT19937_64(0xC5A70000 + k)
    n = rng.choice4(sizes)
    radius = rng.uniform(3.0, 10.0)
    length = rng.uniform(20.0, 100.0)
    a = rng.uniform(20.0, 60.0)
    c = a * rng.uniform(1.0, 1.6)
    sig = rng.uniform(0.05, 0.20)
    azi = rng.uniform(2.0, 20.0)
    return dict(CYL_BCT_FIXED, EditRadius=radius, Length=length, uca=a, ucb=a, ucc=c, EditSigma=sig, SigmaL=sig,
                EditAzi=azi, GridPoints=n // 2, EditPixelNoX=n, EditPixelNoY=n)


def bct_sweep(count=4096):
    return [bct_set(k) for k in range(count)]
