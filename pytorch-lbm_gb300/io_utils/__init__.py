"""Output helpers (the reference's io_utils package): the ASCII VTK writer."""
from .vtk_writer import write_vtk  # noqa: F401
