"""acts_gb300 — GB300-native batched Kalman track fitter (ActsPlugins::CudaKalman)."""
