// runtime_options.cpp -- reader of the H-BLAST_runtime_options text file.
//
// Format (runtime_setting_files/H-BLAST_runtime_options:1-18): nine pairs of
// lines, a comment line followed by a value line, in this order:
// gpu_db_used_ratio, fixed flag, CCR, AVG_HSPS_PER_SEQUENCE, ECC flag,
// balancer method, load factor, chunk size, base value.  Out-of-range values
// fall back the way Read_H_BLAST_runtime_options does
// (NF/functions.cpp:142-202).
#include <stdio.h>
#include <stdlib.h>

#include <string>

#include "../../include/hblast_gpu.h"

namespace {

// Values the reference starts from before reading the file
// (NF/functions.cpp:14-26; h_blast.cu:71 keeps 19+1 HSP slots per subject).
void defaults(hbg_runtime_options *o) {
    o->gpu_db_used_ratio = -1.0;
    o->fixed_ratio = 1;
    o->ccr = 12.0;
    o->avg_hsps_per_sequence = 20;
    o->mem_ecc = 0;
    o->balancer_method = 1;
    o->load_factor = 4;
    o->chunk_size = 200;
    o->base_value = 100;
}

bool read_line(FILE *f, std::string *line) {
    line->clear();
    int c;
    bool any = false;
    while ((c = fgetc(f)) != EOF) {
        any = true;
        if (c == '\n')
            break;
        line->push_back((char)c);
    }
    return any;
}

}  // namespace

extern "C" int hbg_read_runtime_options(const char *path, hbg_runtime_options *o) {
    if (!o)
        return HBG_ERR_INVALID;
    defaults(o);
    if (!path)
        return HBG_OK;
    FILE *f = fopen(path, "rb");
    if (!f)
        return HBG_OK;  // the reference warns and keeps its defaults
    std::string v[9];
    std::string comment;
    int got = 0;
    for (int i = 0; i < 9; ++i) {
        if (!read_line(f, &comment) || !read_line(f, &v[i]))
            break;
        ++got;
    }
    fclose(f);
    if (got > 0) {
        double r = atof(v[0].c_str());
        o->gpu_db_used_ratio = (r < 0 || r > 1) ? 0.0 : r;
    }
    if (got > 1)
        o->fixed_ratio = atoi(v[1].c_str()) == 1 ? 1 : 0;
    if (got > 2) {
        double c = atof(v[2].c_str());
        o->ccr = c <= 0 ? 12.0 : c;
    }
    if (got > 3) {
        int a = atoi(v[3].c_str());
        o->avg_hsps_per_sequence = a > 0 ? a : 20;
    }
    if (got > 4)
        o->mem_ecc = atoi(v[4].c_str()) != 0 ? 1 : 0;
    if (got > 5)
        o->balancer_method = atoi(v[5].c_str()) != 0 ? 1 : 0;
    if (got > 6) {
        int a = atoi(v[6].c_str());
        o->load_factor = a < 0 ? 4 : a;
    }
    if (got > 7) {
        int a = atoi(v[7].c_str());
        o->chunk_size = a < 0 ? 200 : a;
    }
    if (got > 8) {
        int a = atoi(v[8].c_str());
        o->base_value = a < 0 ? 100 : a;
    }
    return HBG_OK;
}
