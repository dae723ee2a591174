// blastdb.h -- reader for NCBI BLAST protein databases (format version 4:
// .pin index + .psq sequences per volume, .pal alias listing volumes).
//
// H-BLAST reads the same files to size its volumes (ExtractVolumeSequences,
// ReadH_BLAST_volinfo; NF/functions.cpp:573-760) and then stages its own
// length-sorted ".hDb" copy written by a patched makeblastdb
// (-sort_volumes, NF/writedb_volume.cpp:255-513; loaded at
// NF/functions.cpp:1058-1165).  Here the .psq bytes are used as they are:
// a .psq is already "0, sequence, 0, sequence, 0 ...", the resident
// database's own layout, so a volume goes to the device as one stream and
// the length schedule is built in memory.
#ifndef HBG_BLASTDB_H
#define HBG_BLASTDB_H

#include <cstdint>
#include <string>
#include <vector>

namespace hbg {

struct BlastDbVolume {
    std::string base;               // path without extension
    std::string title;
    int32_t n = 0;                  // sequences (OIDs)
    int64_t residues = 0;           // sum of sequence lengths
    int32_t max_len = 0;
    int64_t psq_bytes = 0;          // size of the .psq file
    std::vector<uint32_t> seq_off;  // n + 1 offsets into the .psq (big-endian on disk)
};

// Volumes of a database name: `path`.pal (DBLIST, nested aliases allowed) or
// the single volume `path`.pin/.psq.  Returns "" or an error message.
std::string blastdb_volumes(const std::string &path, std::vector<std::string> *volumes);

// Parse and check one volume's .pin (protein, format 4) against its .psq size.
std::string blastdb_read_index(const std::string &base, BlastDbVolume *out);

// Read .psq bytes [from, from + count) into dst and check them: letters
// 1..27 inside sequences, 0 exactly at the separators.  `from` and `count`
// must cover whole sequences plus their separators (the caller walks
// seq_off).
std::string blastdb_read_psq(const BlastDbVolume &v, int64_t from, int64_t count, uint8_t *dst);

}  // namespace hbg

#endif
