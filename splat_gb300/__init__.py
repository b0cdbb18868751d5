"""GB300-native forward trace step of SPLAT (spectral photon-splatting ray tracer)."""
