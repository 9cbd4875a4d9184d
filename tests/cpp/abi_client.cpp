// A C++ caller of the engine's C ABI (include/sph_gb300.h), the way the
// reference's C++ application would drive it: create, initialize, update in
// several calls with the reference's reorder cadence, read the particle
// buffer in the reference's own order, destroy.  Test infrastructure for
// tests/test_gpu_cpp_client.py.
//
//   abi_client <scene.bin> <out.bin>
//
// scene.bin (little endian): 9 float parameters (sph_params order), float dt,
// float reorder interval, uint32 exact, uint32 n, uint32 s, uint32 t,
// uint32 calls, uint32 steps per call, then n*3 floats of positions, s*3
// floats of statics and t*9 floats of triangles.  out.bin: n records of 32
// bytes (sph_dynamic_particle).  Exit status 0 on success.
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_gb300.h"

namespace {

struct Reader {
    FILE* f;
    template <typename T> bool get(T* v, size_t count = 1) { return fread(v, sizeof(T), count, f) == count; }
};

int fail(const char* what, sph_status st)
{
    std::fprintf(stderr, "%s: %s (%s)\n", what, sph_status_string(st), sph_last_error());
    return 1;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 3) { std::fprintf(stderr, "usage: abi_client scene.bin out.bin\n"); return 2; }
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) { std::perror(argv[1]); return 2; }
    Reader r{in};
    sph_params p{};
    float dt = 0.f, interval = 0.f;
    uint32_t exact = 0, n = 0, s = 0, t = 0, calls = 0, steps = 0;
    float raw[9];
    bool ok = r.get(raw, 9) && r.get(&dt) && r.get(&interval) && r.get(&exact) && r.get(&n) && r.get(&s) &&
              r.get(&t) && r.get(&calls) && r.get(&steps);
    std::vector<float> pos(3ull * n), spos(3ull * s), tris(9ull * t);
    ok = ok && r.get(pos.data(), pos.size()) && r.get(spos.data(), spos.size()) && r.get(tris.data(), tris.size());
    std::fclose(in);
    if (!ok) { std::fprintf(stderr, "short scene file\n"); return 2; }
    std::memcpy(&p, raw, sizeof raw);

    sph_engine* e = nullptr;
    sph_status st = sph_engine_create(&e, 0);
    if (st != SPH_OK) return fail("create", st);
    // the reference logs and returns when Update comes before Initialize
    // (SimulationEngineCPU.cpp:422-426); here the call reports it
    if (sph_engine_update(e, dt, 1) != SPH_ERR_NOT_INITIALIZED) {
        std::fprintf(stderr, "update before initialize was not rejected\n");
        return 1;
    }
    st = sph_engine_initialize(e, &p, pos.data(), nullptr, n, s ? spos.data() : nullptr, s,
                               t ? tris.data() : nullptr, t, interval);
    if (st != SPH_OK) return fail("initialize", st);
    if (exact && (st = sph_engine_set_exact(e, 1)) != SPH_OK) return fail("set_exact", st);
    for (uint32_t k = 0; k < calls; ++k)
        if ((st = sph_engine_update(e, dt, steps)) != SPH_OK) return fail("update", st);
    double sim_time = 0.0;
    if ((st = sph_engine_simulation_time(e, &sim_time)) != SPH_OK) return fail("simulation_time", st);
    std::vector<sph_dynamic_particle> outbuf(n);
    if ((st = sph_engine_read_dynamic_buffer(e, outbuf.data())) != SPH_OK) return fail("read", st);
    if ((st = sph_engine_destroy(e)) != SPH_OK) return fail("destroy", st);

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) { std::perror(argv[2]); return 2; }
    const bool wrote = std::fwrite(outbuf.data(), sizeof(sph_dynamic_particle), n, out) == n;
    std::fclose(out);
    std::printf("%s: %u particles, %u calls of %u steps, simulation time %.6f s\n",
                sph_engine_implementation_name(), n, calls, steps, sim_time);
    return wrote ? 0 : 2;
}
