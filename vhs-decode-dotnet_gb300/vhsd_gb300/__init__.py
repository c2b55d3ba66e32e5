"""GB300 (sm_103a) RF decode backend for vhs-decode-dotnet.

``native`` binds the C ABI library (include/vhsdecode_gb300.h), ``backend``
mirrors the reference's managed backend selector and runner for the new
``gb300`` value, ``synth`` generates seeded synthetic RF, ``build`` compiles
the library.
"""
