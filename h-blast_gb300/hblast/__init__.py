"""GB300 word-hit stage (BLASTP/BLASTX): Python binding of include/hblast_gpu.h."""
from .core import (HSP_DTYPE, Batch, Database, GpuOptions, HblastError, ProteinQuery, RuntimeOptions,
                   SearchResult, Searcher, Server, ServerOptions, blastdb_info, blastdb_read, default_options,
                   device_count, fail_allocations, lib, library_path, read_runtime_options, search, seg_mask,
                   seg_params)

__all__ = ["HSP_DTYPE", "Batch", "Database", "GpuOptions", "HblastError", "ProteinQuery", "RuntimeOptions",
           "SearchResult", "Searcher", "Server", "ServerOptions", "blastdb_info", "blastdb_read", "default_options",
           "device_count", "fail_allocations", "lib", "library_path", "read_runtime_options", "search",
           "seg_mask", "seg_params"]
