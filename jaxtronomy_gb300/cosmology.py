"""Background distances for multi-plane ray shooting.

``MultiPlaneBulk`` computes its distance lists on the host, before any GPU
work, from a lenstronomy ``Background`` (lenstronomy >= 1.13.6,
``Cosmo/background.py``) over an astropy cosmology:

* ``d_xy(z1, z2)``: angular diameter distance from z1 to z2 in Mpc, astropy's
  ``angular_diameter_distance_z1z2``;
* ``T_xy(z1, z2) = d_xy(z1, z2) (1 + z2)``: transverse comoving distance in Mpc.

:class:`Background` accepts any object with astropy's
``angular_diameter_distance_z1z2`` method, so an astropy cosmology works
unchanged where astropy is installed.  :class:`FlatLambdaCDM` restates
astropy's ``FlatLambdaCDM(H0, Om0, Tcmb0=0)`` (matter and a cosmological
constant, no radiation) for machines without astropy (Hogg 1999,
arXiv:astro-ph/9905116, eqs. 14-16 and 19):

    E(z) = sqrt(Om0 (1 + z)^3 + 1 - Om0),
    D_C(z1, z2) = (c / H0) int_{z1}^{z2} dz / E(z),
    D_A(z1, z2) = D_C(z1, z2) / (1 + z2)        (flat: D_M = D_C).

The integral is a 64-node Gauss-Legendre rule on [z1, z2]; 1/E is analytic
in a wide ellipse around any interval of z >= 0, so the rule is exact to
rounding.
"""

import numpy as np

C_KM_S = 299792.458  # speed of light [km/s]

_GL_X, _GL_W = np.polynomial.legendre.leggauss(64)


def _value(q):
    """Plain float of an astropy Quantity (its ``.value``) or a number."""
    return float(getattr(q, "value", q))


class FlatLambdaCDM:
    """Flat matter + Lambda cosmology with astropy's distance methods (Mpc floats)."""

    def __init__(self, H0=70.0, Om0=0.3):
        if not (H0 > 0):
            raise ValueError("H0 must be positive")
        if not (0.0 <= Om0 <= 1.0):
            raise ValueError("Om0 must be in [0, 1]")
        self.H0 = float(H0)
        self.Om0 = float(Om0)
        self.Ode0 = 1.0 - self.Om0

    @property
    def hubble_distance(self):
        """c / H0 in Mpc."""
        return C_KM_S / self.H0

    def inv_efunc(self, z):
        z = np.asarray(z, dtype=float)
        return 1.0 / np.sqrt(self.Om0 * (1.0 + z) ** 3 + self.Ode0)

    def comoving_distance_z1z2(self, z1, z2):
        """Line-of-sight comoving distance from z1 to z2 (Mpc)."""
        h = 0.5 * (float(z2) - float(z1))
        m = 0.5 * (float(z2) + float(z1))
        return self.hubble_distance * h * float(np.dot(_GL_W, self.inv_efunc(m + h * _GL_X)))

    def comoving_distance(self, z):
        return self.comoving_distance_z1z2(0.0, z)

    def comoving_transverse_distance(self, z):
        return self.comoving_distance(z)

    def angular_diameter_distance(self, z):
        return self.comoving_distance(z) / (1.0 + float(z))

    def angular_diameter_distance_z1z2(self, z1, z2):
        return self.comoving_distance_z1z2(z1, z2) / (1.0 + float(z2))


class Background:
    """lenstronomy ``Background`` distances over a cosmology object."""

    def __init__(self, cosmo):
        if not hasattr(cosmo, "angular_diameter_distance_z1z2"):
            raise ValueError("cosmo needs an angular_diameter_distance_z1z2(z1, z2) method "
                             "(an astropy cosmology or jaxtronomy_gb300.FlatLambdaCDM)")
        self.cosmo = cosmo

    def d_xy(self, z_observer, z_source):
        """Angular diameter distance between two redshifts (Mpc); elementwise for arrays."""
        zo = np.asarray(z_observer, dtype=float)
        zs = np.asarray(z_source, dtype=float)
        if zo.ndim == 0 and zs.ndim == 0:
            return _value(self.cosmo.angular_diameter_distance_z1z2(float(zo), float(zs)))
        zo, zs = np.broadcast_arrays(zo, zs)
        return np.array([_value(self.cosmo.angular_diameter_distance_z1z2(float(a), float(b)))
                         for a, b in zip(zo.ravel(), zs.ravel())]).reshape(zo.shape)

    def T_xy(self, z_observer, z_source):
        """Transverse comoving distance between two redshifts (Mpc)."""
        return self.d_xy(z_observer, z_source) * (1 + np.asarray(z_source, dtype=float))


def default_background(cosmo=None, cosmology_model="FlatLambdaCDM"):
    """The reference's cosmology choice (``multi_plane_bulk.py:51-55``): the given
    cosmology, else astropy's default (or lenstronomy's ``get_astropy_cosmology``
    for another model name), which need astropy / lenstronomy."""
    if cosmo is None:
        try:
            if cosmology_model == "FlatLambdaCDM":
                from astropy.cosmology import default_cosmology
                cosmo = default_cosmology.get()
            else:
                from lenstronomy.Util.cosmo_util import get_astropy_cosmology
                cosmo = get_astropy_cosmology(cosmology_model=cosmology_model)
        except ImportError as e:
            raise ValueError("cosmo=None selects astropy's default cosmology, and astropy is "
                             "not installed; pass cosmo (an astropy cosmology or "
                             "jaxtronomy_gb300.FlatLambdaCDM(H0, Om0))") from e
    return Background(cosmo)
