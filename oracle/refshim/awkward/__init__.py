"""Import-only stand-in for awkward; the depth>=3 paths it serves are unused."""


def __getattr__(name):
    raise NotImplementedError(f"refshim: awkward.{name} is not available")
