// blastdb.cpp -- NCBI BLAST protein database reader (format 4).
//
// Index file (.pin), every integer big-endian unless noted:
//   u32 format version (4) | u32 type (1 = protein) | u32 title length,
//   title bytes | u32 date length, date bytes | u32 sequence count N |
//   8-byte residue total (NCBI writes it little-endian; both byte orders are
//   accepted when they equal the total the offset table gives) | u32 longest
//   sequence | u32 header offsets[N + 1] | u32 sequence offsets[N + 1].
// The fields up to N are the ones H-BLAST itself parses
// (ExtractVolumeSequences, NF/functions.cpp:573-609).  Sequence file (.psq):
// one 0 byte, then each sequence in NCBIstdaa followed by a 0 byte, so
// sequence i is [off[i], off[i + 1] - 1) and off[N] is the file size.
// Alias file (.pal): text; "DBLIST a b ..." names the volumes (relative to
// the alias file's directory), the way ReadH_BLAST_volinfo reads it
// (NF/functions.cpp:669-760); '#' starts a comment.
#include "blastdb.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <fcntl.h>
#include <sys/stat.h>
#include <thread>
#include <unistd.h>

namespace hbg {

namespace {

constexpr int kAlphabet = 28;   // NCBIstdaa letters 0..27; 0 separates sequences

bool file_size(const std::string &path, int64_t *size) {
    struct stat st;
    if (stat(path.c_str(), &st) != 0 || !S_ISREG(st.st_mode))
        return false;
    *size = (int64_t)st.st_size;
    return true;
}

uint32_t be32(const uint8_t *p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

uint64_t le64(const uint8_t *p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i)
        v = (v << 8) | p[i];
    return v;
}

uint64_t be64(const uint8_t *p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i)
        v = (v << 8) | p[i];
    return v;
}

std::string dir_of(const std::string &path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// Split a DBLIST value: names separated by blanks, a name may be quoted.
std::vector<std::string> split_names(const std::string &s) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r'))
            ++i;
        if (i >= s.size())
            break;
        std::string name;
        if (s[i] == '"') {
            const size_t j = s.find('"', i + 1);
            name = s.substr(i + 1, (j == std::string::npos ? s.size() : j) - i - 1);
            i = j == std::string::npos ? s.size() : j + 1;
        } else {
            size_t j = i;
            while (j < s.size() && s[j] != ' ' && s[j] != '\t' && s[j] != '\r')
                ++j;
            name = s.substr(i, j - i);
            i = j;
        }
        if (!name.empty())
            out.push_back(name);
    }
    return out;
}

std::string volumes_rec(const std::string &path, int depth, std::vector<std::string> *out) {
    if (depth > 8)
        return path + ": alias files nested more than 8 deep";
    int64_t sz = 0;
    const std::string pal = path + ".pal";
    if (!file_size(pal, &sz)) {
        if (!file_size(path + ".pin", &sz))
            return path + ": neither " + path + ".pal nor " + path + ".pin exists";
        out->push_back(path);
        return "";
    }
    std::ifstream in(pal);
    if (!in)
        return pal + ": cannot be read";
    std::string line;
    bool found = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        size_t a = line.find_first_not_of(" \t");
        if (a == std::string::npos || line[a] == '#')
            continue;
        const size_t b = line.find_first_of(" \t", a);
        const std::string key = line.substr(a, b == std::string::npos ? std::string::npos : b - a);
        const std::string rest = b == std::string::npos ? std::string() : line.substr(b);
        if (key == "OIDLIST" || key == "GILIST" || key == "TILIST" || key == "SEQIDLIST" ||
            key == "TAXIDLIST" || key == "FIRST_OID" || key == "LAST_OID")
            return pal + ": " + key + " (a subset of the volumes) is not supported";
        if (key != "DBLIST")
            continue;
        found = true;
        const std::string dir = dir_of(pal);
        for (const std::string &name : split_names(rest)) {
            const std::string vol = (!name.empty() && name[0] == '/') ? name : dir + name;
            std::string err = volumes_rec(vol, depth + 1, out);
            if (!err.empty())
                return err;
        }
    }
    if (!found)
        return pal + ": no DBLIST line";
    return "";
}

}  // namespace

std::string blastdb_volumes(const std::string &path, std::vector<std::string> *volumes) {
    volumes->clear();
    if (path.empty())
        return "empty database name";
    std::string err = volumes_rec(path, 0, volumes);
    if (err.empty() && volumes->empty())
        err = path + ": the alias lists no volumes";
    return err;
}

std::string blastdb_read_index(const std::string &base, BlastDbVolume *out) {
    *out = BlastDbVolume();
    out->base = base;
    const std::string pin = base + ".pin", psq = base + ".psq";
    int64_t pin_size = 0;
    if (!file_size(pin, &pin_size))
        return pin + ": missing";
    if (!file_size(psq, &out->psq_bytes))
        return psq + ": missing";
    std::vector<uint8_t> buf((size_t)pin_size);
    {
        FILE *f = fopen(pin.c_str(), "rb");
        if (!f)
            return pin + ": cannot be opened";
        const size_t got = fread(buf.data(), 1, buf.size(), f);
        fclose(f);
        if ((int64_t)got != pin_size)
            return pin + ": short read";
    }
    size_t at = 0;
    auto need = [&](size_t bytes) { return at + bytes <= buf.size(); };
    const std::string trunc = pin + ": truncated index";
    if (!need(12))
        return trunc;
    const uint32_t version = be32(&buf[0]);
    const uint32_t type = be32(&buf[4]);
    if (version != 4)
        return pin + ": format version " + std::to_string(version) + " (only version 4 is read)";
    if (type != 1)
        return pin + ": not a protein database (type " + std::to_string(type) + ")";
    at = 8;
    const uint32_t title_len = be32(&buf[at]);
    at += 4;
    if (title_len > buf.size() || !need(title_len + 4))
        return trunc;
    out->title.assign(reinterpret_cast<const char *>(&buf[at]), title_len);
    at += title_len;
    const uint32_t date_len = be32(&buf[at]);
    at += 4;
    if (date_len > buf.size() || !need(date_len + 16))
        return trunc;
    at += date_len;
    const uint32_t n = be32(&buf[at]);
    at += 4;
    if (n > 0x7fffffffu)
        return pin + ": sequence count out of range";
    const uint8_t *total_p = &buf[at];
    at += 8;
    const uint32_t max_len = be32(&buf[at]);
    at += 4;
    const size_t table = 4 * ((size_t)n + 1);
    if (!need(2 * table))
        return trunc;
    at += table;                                   // header offsets (.phr): not needed
    out->n = (int32_t)n;
    out->seq_off.resize((size_t)n + 1);
    for (size_t i = 0; i <= n; ++i)
        out->seq_off[i] = be32(&buf[at + 4 * i]);
    // consistency: offsets start after the leading 0, every sequence is
    // followed by a separator, and the table ends at the end of the .psq
    if (out->seq_off[0] != 1)
        return pin + ": first sequence offset is " + std::to_string(out->seq_off[0]) + ", not 1";
    if ((int64_t)out->seq_off[n] != out->psq_bytes)
        return pin + ": sequence offsets end at " + std::to_string(out->seq_off[n]) + " but " + psq +
               " has " + std::to_string(out->psq_bytes) + " bytes";
    int64_t total = 0;
    int32_t longest = 0;
    for (size_t i = 0; i < n; ++i) {
        if (out->seq_off[i + 1] <= out->seq_off[i])
            return pin + ": sequence offsets are not increasing at " + std::to_string(i);
        const int64_t L = (int64_t)out->seq_off[i + 1] - out->seq_off[i] - 1;
        total += L;
        longest = std::max<int32_t>(longest, (int32_t)L);
    }
    if (le64(total_p) != (uint64_t)total && be64(total_p) != (uint64_t)total)
        return pin + ": residue total does not match the offset table";
    if ((int32_t)max_len != longest)
        return pin + ": longest-sequence field does not match the offset table";
    out->residues = total;
    out->max_len = longest;
    return "";
}

std::string blastdb_read_psq(const BlastDbVolume &v, int64_t from, int64_t count, uint8_t *dst) {
    const std::string psq = v.base + ".psq";
    if (from < 0 || count < 0 || from + count > v.psq_bytes)
        return psq + ": read outside the file";
    const int fd = open(psq.c_str(), O_RDONLY);
    if (fd < 0)
        return psq + ": cannot be opened";
    // large reads are split over a few threads, each reading (pread) and
    // checking its share: letters in range and the number of 0 bytes
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = count >= (8 << 20) ? (int)std::min(8u, hw) : 1;
    std::vector<int64_t> zeros_t(nt, 0);
    std::vector<int> bad_t(nt, 0);         // 1 short read, 2 letter out of range
    auto work = [&](int t) {
        const int64_t lo = count * t / nt, hi = count * (t + 1) / nt;
        int64_t at = lo;
        while (at < hi) {
            const ssize_t r = pread(fd, dst + at, (size_t)(hi - at), (off_t)(from + at));
            if (r <= 0) {
                bad_t[t] = 1;
                return;
            }
            at += r;
        }
        // 4 KiB blocks with narrow accumulators (the compiler vectorises these)
        uint32_t above = 0;
        int64_t zeros = 0;
        for (int64_t b = lo; b < hi; b += 4096) {
            const int64_t e = std::min<int64_t>(b + 4096, hi);
            uint8_t ab = 0;
            uint32_t z = 0;
            for (int64_t i = b; i < e; ++i) {
                ab |= (uint8_t)(dst[i] >= kAlphabet);
                z += dst[i] == 0;
            }
            above |= ab;
            zeros += z;
        }
        zeros_t[t] = zeros;
        if (above)
            bad_t[t] = 2;
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back(work, t);
        for (std::thread &x : th)
            x.join();
    }
    close(fd);
    int64_t zeros = 0;
    for (int t = 0; t < nt; ++t) {
        if (bad_t[t] == 1)
            return psq + ": short read";
        if (bad_t[t] == 2)
            return psq + ": letter outside NCBIstdaa 0..27";
        zeros += zeros_t[t];
    }
    int64_t seps = 0;
    if (from == 0) {
        if (count > 0 && dst[0] != 0)
            return psq + ": does not start with a 0 byte";
        seps += count > 0;
    }
    // separators inside [from, from + count): the bytes off[i] - 1 for i >= 1
    auto lo = std::lower_bound(v.seq_off.begin() + 1, v.seq_off.end(), (uint32_t)(from + 1));
    for (auto it = lo; it != v.seq_off.end() && (int64_t)*it - 1 < from + count; ++it) {
        if (dst[(int64_t)*it - 1 - from] != 0)
            return psq + ": sequence not followed by a 0 byte";
        ++seps;
    }
    if (zeros != seps)
        return psq + ": a 0 byte inside a sequence";
    return "";
}

}  // namespace hbg
