"""fairsim-vigor_gb300: GB300-native (sm_103a) 2D SIM reconstruction behind fairSIM's API."""
from .sim_param import Dir, OtfProvider, SimParam  # noqa: F401
from . import synth  # noqa: F401
