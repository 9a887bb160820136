"""GB300-native timestep engine for ProjecTracer-style tracer convection (see include/ptgpu.h)."""
