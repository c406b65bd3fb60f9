"""Write include/mocca_gpu.f90, the iso_c_binding module of the C header
include/mocca_gpu.h for a Fortran host: one bind(C) derived type per struct
and one interface per entry point (values and c_ptr arguments), plus
gpu_check (negative status -> the reference's stp()).  Run after changing
the header:
    python include/make_fortran_module.py
tests/test_abi.py checks that the committed module is what this writes.
"""
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

HEAD = """! mocca_gpu.f90 -- iso_c_binding interface of libmocca_gpu (include/mocca_gpu.h)
! for the Fortran host: one bind(C) derived type per struct of the C header
! and one interface per entry point.  Every argument crosses as a value or a
! c_ptr: pass c_loc() of a scalar, array or derived-type variable, and an
! array of c_ptr for the lists of grids (one c_loc(HFBasis(i)%Value%Grid)
! per spwf).  Every function returns the status of the C header (0 ok,
! > 0 not converged, < 0 error); gpu_check turns an error into the
! reference's stp().  Written by include/make_fortran_module.py.
"""

TAIL = """contains
  subroutine gpu_check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st .lt. 0) call stp('mocca_gpu call failed: ' // where, 'status', int(st))
  end subroutine gpu_check
end module mocca_gpu
"""

FTYPE = {"int": "integer(c_int)", "double": "real(c_double)"}


def module_text(header: str) -> str:
    src = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    out = [HEAD.rstrip("\n"),
           "module mocca_gpu\n  use iso_c_binding\n  use GenInfo, only : stp\n  implicit none\n"]
    for name, body in re.findall(r"typedef struct (\w+) \{(.*?)\} \w+;", src, flags=re.S):
        out.append(f"  type, bind(C) :: {name}")
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(int|double)\s+(.*)", decl)
            for var in (v.strip() for v in m.group(2).split(",")):
                dims = re.findall(r"\[(\d+)\]", var)
                vname = var.split("[")[0]
                # C row-major [a][b] is Fortran column-major (b, a)
                shape = f"({','.join(reversed(dims))})" if dims else ""
                out.append(f"    {FTYPE[m.group(1)]} :: {vname}{shape}")
        out.append(f"  end type {name}")
    out.append("\n  interface")
    for fn, args in re.findall(r"^int\s+(mg_\w+)\s*\((.*?)\);", src, flags=re.S | re.M):
        names, decls = [], []
        for a in (x.strip() for x in " ".join(args.split()).split(",")):
            m = re.match(r"(const\s+)?([\w ]+?)\s*(\*+(?:\s*const\s*\*)?)?\s*(\w+)$", a)
            base, stars, an = m.group(2).strip(), (m.group(3) or "").replace(" ", ""), m.group(4)
            names.append(an)
            if stars in ("**", "*const*") and base in ("mg_ctx", "mg_batch"):
                decls.append(f"type(c_ptr), intent(out) :: {an}")   # handle returned
            elif stars:
                decls.append(f"type(c_ptr), value :: {an}")
            else:
                decls.append(f"{FTYPE[base]}, value :: {an}")
        out.append(f'    integer(c_int) function {fn}({", ".join(names)}) bind(C, name="{fn}")')
        out.append("      import")
        out += [f"      {d}" for d in decls]
        out.append("    end function")
    out.append("  end interface")
    return "\n".join(out) + "\n" + TAIL


if __name__ == "__main__":
    text = module_text((HERE / "mocca_gpu.h").read_text())
    (HERE / "mocca_gpu.f90").write_text(text)
    sys.stdout.write(f"wrote {HERE / 'mocca_gpu.f90'}\n")
