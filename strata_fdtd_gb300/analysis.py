"""Frequency weighting and sound levels under the reference's analysis
module name (analysis/weighting.py of rjwalters/strata-fdtd)."""
from .weighting import (P_REF, apply_weighting, calculate_leq, calculate_spl,  # noqa: F401
                        calculate_time_weighted_level, get_weighting_sos,
                        weighting_response)
