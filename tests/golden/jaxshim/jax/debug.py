"""jax.debug of the numpy stand-in."""


def print(*a, **k):  # noqa: A001
    pass


def callback(fn, *a, **k):
    fn(*a)
