// moqui's own input-file reader (mqi::file_parser, moqui/base/mqi_file_handler.hpp:220-420) on a
// file, for the parser tests: test infrastructure, compiled from the staged reference headers
// (oracle/stage_ref.py stages the reader without its DICOM includes).
//
//   ref_parser <input file> <query>...      query: <type>:<key>:<default>
//
// type s: get_string, f: get_float (printed with 9 significant digits), i: get_int, b: get_bool
// (printed 0 / 1), v: get_string_vector with "," (the items joined by '|').  One output line per
// query.  When the reader throws (a line or a value of white space only), the message goes to
// stderr and the exit status is 3.
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
