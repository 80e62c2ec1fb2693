"""caustics_gb300: GB300-native (sm_103a) magnification hot path of
fbartolic/caustics — Ehrlich-Aberth root solver, point-source and
extended-source (contour-integration) magnification, hexadecapole routing —
behind a C ABI (include/caustics_gb300.h) with the reference's Python
signatures, and as torch operators (torch.ops.caustics.*, caustics_gb300.ops)."""
from . import ops  # noqa: F401  (registers the torch operators)
from .api import (  # noqa: F401
    AnnualParallaxTrajectory,
    BatchedLightCurves,
    ExtendedSourceMagnification,
    LightCurveLogLikelihood,
    LightCurveMagnification,
    critical_and_caustic_curves,
    ehrlich_aberth,
    mag_extended_source_grad,
    mag_lc_batched,
    mag_lc_batched_vjp,
    lens_eq,
    lens_eq_det_jac,
    lens_polynomial,
    mag,
    mag_extended_source,
    mag_point_source,
    marginalized_log_likelihood,
    marginalized_log_likelihood_batched,
    poly_roots,
    project_onto_sky,
    roots_jvp,
    roots_vjp,
)

__all__ = ["ehrlich_aberth", "poly_roots", "lens_polynomial", "lens_eq", "lens_eq_det_jac", "mag_point_source", "mag_extended_source",
           "mag", "mag_extended_source_grad", "mag_lc_batched", "mag_lc_batched_vjp", "LightCurveMagnification", "BatchedLightCurves",
           "roots_jvp", "roots_vjp", "critical_and_caustic_curves",
           "marginalized_log_likelihood", "marginalized_log_likelihood_batched", "LightCurveLogLikelihood",
           "AnnualParallaxTrajectory", "ExtendedSourceMagnification", "project_onto_sky"]
