"""pypty_gb300: the far-field multislice ptychography hot path of pypty on one GB300.

Layers (top to bottom):
  objective.loss_and_direction  drop-in for pypty.objective.loss_and_direction
  fft                           drop-in window FFT wrappers (pypty.fft)
  shim.install                  installs the drop-ins into an imported pypty package
  engine.Engine                 device-resident calls with torch tensors
  _lib                          ctypes binding of include/pypty_gb300.h
  csrc/                         CUDA kernels for sm_103a and the C ABI
"""
__version__ = "0.1.0"
