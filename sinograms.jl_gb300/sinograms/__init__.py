"""sinograms -- host-side mirror of the Sinograms.jl API over libsinogb300.so.

Names, argument meaning and error behaviour follow the reference package
(JuliaImageRecon/Sinograms.jl v0.5.1); every computation runs in the CUDA library
(include/sinogb300.h).  See geom.py for the array-order convention.
"""
from ._lib import SinogramsError, launch_count, measure_peaks
from .bdd import BddGeo, BddPlan, backproject_bdd, project_bdd
from .filters import (SinogramsArgumentError, Window, _angle_weights, fbp_filter, fbp_ramp, fbp_sino_filter,
                      fbp_sino_weight, fbp_window, fdk_view_weight, fbp_view_weight, fdk_weight_cyl, parker_weight,
                      ramp_arc, ramp_flat)
from .footprint import footprint_size, zwart_powell, zwart_powell_sino
from .geom import (CtFanArc, CtFanFlat, CtPar, CtSourceCircle, CtSourceHelix, ImageGeom, SinoFanArc, SinoFanFlat, SinoMoj, SinoPar, _ar, _d_ang, _dso, _gamma, _gamma_max, _source_dz_per_view, _source_zs, _zfov,
                   _orbit_short, _rfov, _s, _t, angles, axes, dims, downsample)
from .phantoms import ellipse_sino, ellipsoid_proj, random_ct_scans, random_ellipses, random_ellipsoids
from .sf import SFPlan, _tau, backproject_sf, project_sf
from .recon import FBPNormalPlan, FDKBatch, FDKplan, cbct_back, fbp, fbp_back, fdk, plan_fbp

__all__ = [n for n in dir() if not n.startswith("__")]
