"""Front-end compatibility shim for running OpenSBLI's problem definitions on current SymPy.

OpenSBLI pins SymPy 1.1 (environment_and_run_scripts/InstallPython.sh:50) and assigns
``Indexed.is_commutative`` per instance (opensbli/core/opensblifunctions.py:31), which later
SymPy versions expose as a read-only property.  ``apply()`` makes that attribute settable per
instance again; nothing else about SymPy changes.  Call it before building the problem.
"""


def apply():
    import sympy
    from sympy import Indexed
    if getattr(Indexed, "_osb_settable_commutative", False):
        return
    base = sympy.Basic.is_commutative

    def _get(self):
        d = getattr(self, "__dict__", None)
        if d is not None and "_osb_is_comm" in d:
            return d["_osb_is_comm"]
        return base.fget(self)

    def _set(self, value):
        self.__dict__["_osb_is_comm"] = value

    Indexed.is_commutative = property(_get, _set)
    Indexed._osb_settable_commutative = True
