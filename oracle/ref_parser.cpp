// moqui's own input-file and mask readers (mqi::file_parser and mqi::mask_reader,
// moqui/base/mqi_file_handler.hpp:13-420) on files, for the parser tests: test infrastructure,
// compiled from the staged reference headers (oracle/stage_ref.py stages the readers without their
// DICOM includes).
//
//   ref_parser <input file> <query>...      query: <type>:<key>:<default>
//   ref_parser --mask <nx> <ny> <nz> <mask.mha>...
//
// type s: get_string, f: get_float (printed with 9 significant digits), i: get_int, b: get_bool
// (printed 0 / 1), v: get_string_vector with "," (the items joined by '|').  One output line per
// query.  When the reader throws (a line or a value of white space only), the message goes to
// stderr and the exit status is 3.
//
// --mask: mask_reader::read_mask_files (the masks summed) and mask_to_roi (the CONTOUR runs); prints
// "roi <length>" and one line per run, "run <start> <stride> <accumulated stride>", or "run <start>
// open" for a run that no voxel of sum 0 closes before the end of the volume (moqui leaves its
// stride unset).
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include <moqui/base/mqi_file_handler_parser.hpp>

int
main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_parser <input file> <type:key:default>...\n");
        return 2;
    }
    if (std::string(argv[1]) == "--mask") {
        if (argc < 6) return 2;
        try {
            const int                nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
            std::vector<std::string> files(argv + 5, argv + argc);
            mqi::mask_reader         mr(files, mqi::vec3<mqi::ijk_t>(nx, ny, nz));
            mr.read_mask_files();
            const mqi::roi_t* roi = mr.mask_to_roi();
            std::printf("roi %u\n", roi->length_);
            const size_t n = (size_t) nx * ny * nz;
            for (uint32_t k = 0; k < roi->length_; ++k) {
                bool closed = false;
                for (size_t v = roi->start_[k]; v < n && !closed; ++v) closed = mr.mask_total[v] == 0;
                if (closed) std::printf("run %u %u %u\n", roi->start_[k], roi->stride_[k], roi->acc_stride_[k]);
                else std::printf("run %u open\n", roi->start_[k]);
            }
        } catch (const std::exception& e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 3;
        }
        return 0;
    }
    try {
        mqi::file_parser p(argv[1], " ");
        for (int i = 2; i < argc; ++i) {
            const std::string q = argv[i];
            const size_t      a = q.find(':', 2);
            if (q.size() < 3 || q[1] != ':' || a == std::string::npos) {
                std::fprintf(stderr, "bad query: %s\n", argv[i]);
                return 2;
            }
            const std::string key = q.substr(2, a - 2), dflt = q.substr(a + 1);
            switch (q[0]) {
            case 's': std::printf("%s\n", p.get_string(key, dflt).c_str()); break;
            case 'f': std::printf("%.9g\n", p.get_float(key, (float) std::atof(dflt.c_str()))); break;
            case 'i': std::printf("%d\n", p.get_int(key, std::atoi(dflt.c_str()))); break;
            case 'b': std::printf("%d\n", (int) p.get_bool(key, std::atoi(dflt.c_str()) != 0)); break;
            case 'v': {
                const std::vector<std::string> v = p.get_string_vector(key, ",");
                std::string                    out;
                for (size_t k = 0; k < v.size(); ++k) out += (k ? "|" : "") + v[k];
                std::printf("%s\n", out.c_str());
                break;
            }
            default: std::fprintf(stderr, "bad query type: %s\n", argv[i]); return 2;
            }
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
