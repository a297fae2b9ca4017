"""No-op stand-in for colorama (oracle test infrastructure only)."""


def init(*args, **kwargs):
    pass


class _Codes:
    def __getattr__(self, name):
        return ""


Fore = _Codes()
Back = _Codes()
Style = _Codes()
