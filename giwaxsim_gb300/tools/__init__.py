"""Drop-in replacements for the reference's tools/ modules, backed by the
GB300 native library (giwaxsim_gb300/_lib/libgiwaxs_gb300.so)."""
