"""GB300-native LETKF analysis: the host side of the reference's letkf_run."""
