from invoke.vendor.yaml import *  # noqa: F401,F403
from invoke.vendor.yaml import safe_load  # noqa: F401
