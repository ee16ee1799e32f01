"""Stand-in for cupy.cuda: one device with one SM, synchronous streams."""


class _Stream:
    def synchronize(self):
        return None


class Stream:
    null = _Stream()


def get_current_stream():
    return Stream.null


class Device:
    def __init__(self, device_id=0):
        self.id = device_id
        self.attributes = {"MultiProcessorCount": 1}

    def synchronize(self):
        return None


class runtime:  # noqa: N801 - mirrors cupy.cuda.runtime module access
    @staticmethod
    def getDeviceProperties(dev_id):
        return {"name": b"refshim-cpu"}

    @staticmethod
    def getDeviceCount():
        return 1
