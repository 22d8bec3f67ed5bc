"""GB300 (sm_103a) implementation of the ALBATROS baseband hot path:
4-bit / 1-bit unpack -> inverse PFB -> forward PFB re-channelisation ->
time-averaged cross-correlation, behind the call surface of
PhilJ0ly/albatros_axion_detection (albatros_analysis/src).

Modules mirror the reference's:
  unpacking              unpack_4bit, unpack_1bit, sortpols, hist
  baseband_data_classes  make_continuous_gpu
  pfb_gpu_utils          sinc_hamming, get_matft, calculate_filter, cupy_ipfb, cupy_pfb
  correlations           avg_xcorr_all_ant_gpu, avg_xcorr_4bit(_2ant), avg_xcorr_1bit(...),
                         van_vleck_correction, xcorr_coarse_4bit
  stream                 ProcessingConfig, JobChunkPlanner, StreamCorrelator, repfb_xcorr_avg
  ingest                 read_header, get_header, BasebandFileIterator, file-level repfb_xcorr_avg
  output                 missing_fraction, mask_invalid, save_xcorr_npz, write_run
and two have no reference counterpart:
  batch                  BatchCorrelator: many files of mixed format in one CUDA graph
  autotune               time-stage form, tile and FFT radix order per configuration

All compute runs in the CUDA library lib/libalbatros_gb300.so (C-ABI in
include/albatros_gb300.h); there is no CPU fallback.
"""
from . import _lib  # noqa: F401

__version__ = "0.1.0"
