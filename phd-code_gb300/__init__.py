"""GB300-native flux path for the AREPO-style moving-mesh code rickyfernandez/phd-code.

Importable as ``phd_code_gb300`` (the directory name carries a hyphen; see
``__graft_entry__.load_package``).
"""
__version__ = "0.1.0"
