"""Import placeholder (test infrastructure only); attributes resolve to a dummy."""


class _Dummy:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Dummy()

    def __getattr__(self, name):
        return _Dummy()


def __getattr__(name):
    return _Dummy()
