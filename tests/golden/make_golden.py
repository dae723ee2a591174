"""Regenerate tests/golden/reference_tables.json from the H-BLAST tree.

Run with HBLAST_REFERENCE set to the root of a checkout of the H-BLAST
repository (the directory that holds h_blast_v1.1/); tests only read the
committed JSON.  What is extracted, and from where (paths inside the reference):
  - the BLOSUM62 table over NCBIstdaa, h_blast_v1.1/H-BLAST/h_blast.c:42-71
  - word-index constants CHARSIZE and AA_HITS_PER_CELL,
    h_blast_kernel.cu:1-3 and h_blast_kernel.h:39
  - the default -gpu_threads / -gpu_blocks values, ncbi_blast_files/gpu_cpu_common.h:12,14
  - the shipped runtime-options file, runtime_setting_files/H-BLAST_runtime_options
"""
from __future__ import annotations

import json
import os
import re
from pathlib import Path

OUT = Path(__file__).resolve().parent / "reference_tables.json"


def main() -> None:
    root = os.environ.get("HBLAST_REFERENCE")
    if not root:
        raise SystemExit("set HBLAST_REFERENCE to the root of an H-BLAST checkout")
    REF = Path(root) / "h_blast_v1.1"
    HB = REF / "H-BLAST"
    src = (HB / "h_blast.c").read_text()
    body = src[src.index("Blosum62[28][32]"):]
    rows = re.findall(r"\{([-\d,\s]+)\}", body)[:28]
    matrix = [[int(x) for x in r.split(",")] for r in rows]
    assert len(matrix) == 28 and all(len(r) == 32 for r in matrix)
    kern = (HB / "h_blast_kernel.cu").read_text()
    charsize = int(re.search(r"#define\s+CHARSIZE\s+(\d+)", kern).group(1))
    khdr = (HB / "h_blast_kernel.h").read_text()
    hits_per_cell = int(re.search(r"#define\s+AA_HITS_PER_CELL\s+(\d+)", khdr).group(1))
    common = (HB / "ncbi_blast_files" / "gpu_cpu_common.h").read_text()
    threads = int(re.search(r"#define\s+NUM_THREADSX\s+(\d+)", common).group(1))
    blocks = int(re.search(r"#define\s+NUM_BLOCKSX\s+(\d+)", common).group(1))
    runtime = (REF / "runtime_setting_files" / "H-BLAST_runtime_options").read_text()
    text = json.dumps({
        "source": "H-BLAST v1.1 (h_blast_v1.1/H-BLAST)",
        "blosum62_ncbistdaa_28x32": ["@ROW%d@" % i for i in range(28)],
        "charsize": charsize,
        "aa_hits_per_cell": hits_per_cell,
        "default_gpu_threads": threads,
        "default_gpu_blocks": blocks,
        "runtime_options_file": runtime,
    }, indent=1)
    for i, r in enumerate(matrix):       # one matrix row per line
        text = text.replace('"@ROW%d@"' % i, json.dumps(r))
    OUT.write_text(text + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
