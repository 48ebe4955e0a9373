"""GB300-native drop-in for the reference's ``xpbd_gpu`` package.

``xpbd_gpu.neohookean_solver.XPBDNeoHookeanSolver`` and ``xpbd_gpu.sdf`` keep
the reference's class interface; the substep runs as hand-written sm_103a CUDA
kernels in ``libxpbd_gb300.so`` reached through a ctypes C ABI
(``include/xpbd_gb300.h``).  There is no CPU fallback.
"""
