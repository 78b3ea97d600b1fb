"""phys-engine-gb300: the per-step collision-and-contact path of bkuangs/phys-engine's
PhysicsWorld::step(dt), rebuilt as hand-written CUDA kernels for GB300 (sm_103a)
behind a C ABI (include/phys_gb300.h).  This Python package is a thin ctypes
binding used by the tests and the benchmark; the engine itself is native code."""
