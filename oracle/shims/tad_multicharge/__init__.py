"""Import-time stand-in for tad-multicharge 0.5.0.  TEST INFRASTRUCTURE ONLY.
The oracle uses the SAD (zero-charge) guess, so EEQ is never called."""


def get_eeq_charges(*args, **kwargs):
    raise NotImplementedError("EEQ guess not available; use guess='sad'")
