"""Comparator arms of the benchmark (never imported by the product package).

``plain_gpu``: the reference's plain GPU path of the streaming chain, its CuPy
glue restated in torch around a cuFFT / cuBLAS shim (``plain_gpu_shim.cu``).
"""
