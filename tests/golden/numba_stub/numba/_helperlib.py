"""Stub of numba._helperlib: imported by the reference at module load; its
random-state functions are never called by the fixture generator."""


def _unused(*a, **k):
    raise NotImplementedError("numba stub: random-state helpers are not available")


rnd_get_np_state_ptr = rnd_get_state = rnd_set_state = _unused
