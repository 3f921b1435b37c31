"""Build recipe of the oracle's C/OpenMP restatement (test infrastructure;
output under oracle/_build/, which stays out of the commits)."""
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build" / "libicp_port.so"
# -ffp-contract=off: no fused multiply-add, so float32 results equal the
# numpy oracle's bit for bit on x86 and on Arm alike.
FLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
         "-D_GNU_SOURCE"]


def build():
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / "icp_port.c"
    if OUT.exists() and OUT.stat().st_mtime > src.stat().st_mtime:
        return OUT
    subprocess.run(["gcc", *FLAGS, str(src), "-o", str(OUT), "-lm"], check=True)
    return OUT


def load():
    import ctypes
    lib = ctypes.CDLL(str(build()))
    vp, i64, i32, f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
    lib.icp_port_estimate.restype = ctypes.c_int
    lib.icp_port_estimate.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp, vp, i32, i32, vp, i32,
                                      vp, i32, f64, f64, f64, f64, f64, i32, vp, vp, vp, vp, vp]
    lib.icp_port_max_threads.restype = ctypes.c_int
    return lib


if __name__ == "__main__":
    print(build())
