from . import EV2AU, KELVIN2AU, AU2EV  # noqa: F401
