"""GB300-native rebuild of wendy's approximate 1D N-body integrator."""
