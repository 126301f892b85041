"""Exception classes; the first two keep the names of the reference's
(hmclab/Helpers/CustomExceptions.py:4-21)."""


class AbstractMethodError(Exception):
    """Raised when an abstract method of a plugin class is called."""

    def __init__(self):
        super().__init__("This method is abstract and should be implemented by a derived class.")


class InvalidCaseError(Exception):
    """Raised when a request is valid in general but not for this instance."""


class DeviceUnavailableError(RuntimeError):
    """The CUDA library or a CUDA device is missing.  hmclab_gb300 computes on
    the GPU only; there is no CPU fallback."""


class DeviceTimeoutError(RuntimeError):
    """A bounded wait inside a device kernel ran out; the kernel returned
    without completing its work and the context stays usable."""
