"""Test infrastructure: builds the reference's own registration sources into
``oracle/_ref/`` (a torch extension module, ``slamtb_ref``), so that the CPU
tests can run the reference's code on the same inputs as the oracle.

Recipe (nothing is copied; the sources are compiled where they lie):

* ``src/correspondence_map.cu``, ``src/icp_jacobian_geometric.cu``,
  ``src/icp_jacobian_feature.cu``, ``src/merge_map.cpp``,
  ``src/cuda_utils.cpp`` and the frame preparation (``src/normals.cu``,
  ``src/downsample.cu``, ``src/erode_mask.cu``,
  ``src/bilateral_depth_filter.cu``) of the reference, with its
  ``include/slamtb`` and ``src`` directories on the include path;
* ``oracle/ref_shim`` first on the include path: the project's subset of
  Eigen (the reference needs Eigen >= 3.3.7, which this image lacks) and an
  empty ``pybind11/eigen.h`` (included by ``icp_jacobian_feature.cu`` for
  bindings it does not define);
* ``oracle/ref_binding.cpp``: the module's Python binding.

The reference's own build (CMake + FindCUDA, ``setup.py``) is not used.
Without ``NDEBUG`` the reference's CPU loops run sequentially
(``kernel.hpp``: OpenMP only under NDEBUG), so its CPU correspondence map
keeps, among equal distances, the first writer: the smallest source index.

The reference tree is looked up in ``$SLAMTB_REFERENCE``; ``build()``
returns None when it is absent (the GPU machine has no copy of it).
"""
import os
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_ref"
SOURCES = ["src/correspondence_map.cu", "src/icp_jacobian_geometric.cu",
           "src/icp_jacobian_feature.cu", "src/merge_map.cpp", "src/cuda_utils.cpp",
           "src/normals.cu", "src/downsample.cu", "src/erode_mask.cu",
           "src/bilateral_depth_filter.cu"]


def reference_root():
    p = os.environ.get("SLAMTB_REFERENCE")
    return pathlib.Path(p) if p else None


def build(verbose=False):
    """Compiles (or loads the up-to-date build of) the reference module;
    returns the module, or None without a reference tree."""
    ref = reference_root()
    if ref is None or not all((ref / s).exists() for s in SOURCES):
        return None
    os.environ.setdefault("TORCH_CUDA_ARCH_LIST", "10.0")
    from torch.utils.cpp_extension import load
    OUT.mkdir(exist_ok=True)
    return load(
        name="slamtb_ref",
        sources=[str(HERE / "ref_binding.cpp")] + [str(ref / s) for s in SOURCES],
        extra_include_paths=[str(HERE / "ref_shim"), str(ref / "include" / "slamtb"),
                             str(ref / "src")],
        # the reference's headers forward-declare pybind11::module, which
        # torch/extension.h (pulled into torch/torch.h by this define)
        # defines otherwise
        extra_cflags=["-O2", "-UTORCH_API_INCLUDE_EXTENSION_H"],
        extra_cuda_cflags=["-O2", "-UTORCH_API_INCLUDE_EXTENSION_H"],
        build_directory=str(OUT),
        verbose=verbose)


def load():
    """The reference module: the build under ``oracle/_ref/`` when present
    (no reference tree needed), else a fresh build; None when neither is
    possible."""
    so = OUT / "slamtb_ref.so"
    if so.exists():
        import importlib.machinery
        import importlib.util

        import torch  # noqa: F401  (the module links against torch's libraries)
        loader = importlib.machinery.ExtensionFileLoader("slamtb_ref", str(so))
        spec = importlib.util.spec_from_file_location("slamtb_ref", str(so), loader=loader)
        try:
            mod = importlib.util.module_from_spec(spec)
            loader.exec_module(mod)
            return mod
        except ImportError:
            pass  # built for another machine or torch: rebuild below
    return build()


if __name__ == "__main__":
    print(build(verbose=True))
