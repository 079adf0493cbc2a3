// moqui's phantom example (tests/mc/phantom/phantom_env.cpp) with phantom_env_gb300: the same
// command line and output files, the transport on libmqigpu.so.  Built against moqui's headers:
//   g++ -std=c++17 -O2 [-D__PHYSICS_DEBUG__] -I<moqui root> -I<this repo>/include \
//       -I<this directory> phantom_env_gb300_main.cpp -L<lib dir> -lmqigpu -lz
#include <chrono>
#include <cstdio>

#include "mqi_phantom_env_gb300.hpp"

// moqui's print_materials reads material members that no longer exist
// (moqui/kernel_functions/mqi_print_data.hpp:20-24), so its host instantiation does not compile;
// an empty specialisation stands in for the diagnostic printout.
template<>
void
mc::print_materials<float>(mqi::material_t<float>*, uint16_t) {}

int
main(int argc, char* argv[]) {
    try {
        mqi::cli cl_opts;
        cl_opts.read(argc, argv);
        phantom_env_gb300<float> env(cl_opts);
        env.initialize();
        const auto t0 = std::chrono::steady_clock::now();
        env.run();
        const auto t1 = std::chrono::steady_clock::now();
        env.finalize();
        env.save_reshaped_files();
        std::printf("transport %.6f s\n", std::chrono::duration<double>(t1 - t0).count());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "phantom_env_gb300: %s\n", e.what());
        return 1;
    }
    return 0;
}
