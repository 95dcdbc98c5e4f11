// fdtd_main.cpp -- drop-in replacement for the reference program (fdtd.cu:46-544).
//
// Reads the same files (input_params, mat_specs, v1_%05d.pgm slices), runs
// iterationsCount steps (t_max rounded up to a multiple of 3) and, like the
// reference, writes all nine fields every step in the writeResults3d layout
// under output_dir.  The set-up order of the reference is kept: the Mur
// slabs come from the default material of input_params (fdtd.cu:59 runs
// before loadMaterials at :65).
//
// Options (none changes the reference behaviour unless given):
//   --params PATH        input_params file        (default data/input_params)
//   --specs PATH         mat_specs file           (default data/mat_specs_riken)
//   --scheme reference|corrected
//   --every N            snapshot period in steps (default 1; 0 = no output)
//   --fields LIST        e.g. ex,ey,ez            (default all nine)
//   --format text|binary|both
//                        reference text layout (default), raw float32 files, or both
//   --timeskip X         dt factor                (default 1.0, as the reference)
//   --kernel single|two|compact
//                        fused single-pass, two-pass, or the single-pass compact
//                        form (nine stored fields: D is not written)
//   --voxel-cache PATH   read the class volume from a binary cache made by an
//                        earlier run, or parse the slices and write it
//   --device N
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fdtd_gb300.h"

namespace {

int fail(const char *what, int st)
{
    std::fprintf(stderr, "fdtd: %s failed: %s (%d)\n", what, fdtd_status_string(st), st);
    return 1;
}

uint32_t parse_fields(const std::string &list)
{
    static const char *names[FDTD_FIELD_COUNT] = {"hx", "hy", "hz", "dx", "dy", "dz", "ex", "ey", "ez"};
    uint32_t mask = 0;
    size_t pos = 0;
    while (pos <= list.size()) {
        const size_t end = list.find(',', pos);
        const std::string tok = list.substr(pos, end == std::string::npos ? std::string::npos : end - pos);
        for (int f = 0; f < FDTD_FIELD_COUNT; f++)
            if (tok == names[f])
                mask |= 1u << f;
        if (end == std::string::npos)
            break;
        pos = end + 1;
    }
    return mask;
}

}  // namespace

int main(int argc, char **argv)
{
    std::string params_path = "data/input_params", specs_path = "data/mat_specs_riken", voxel_cache;
    int scheme = FDTD_SCHEME_REFERENCE, every = 1, device = 0, kernel = FDTD_KERNEL_SINGLE_PASS;
    int format = FDTD_SNAPSHOT_TEXT;
    uint32_t mask = (1u << FDTD_FIELD_COUNT) - 1;
    float timeskip = 1.0f;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto next = [&]() -> const char * {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "fdtd: %s needs a value\n", a.c_str());
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--params") params_path = next();
        else if (a == "--specs") specs_path = next();
        else if (a == "--scheme") scheme = std::strcmp(next(), "corrected") == 0 ? FDTD_SCHEME_CORRECTED : FDTD_SCHEME_REFERENCE;
        else if (a == "--every") every = std::atoi(next());
        else if (a == "--fields") mask = parse_fields(next());
        else if (a == "--format") {
            const char *f = next();
            format = std::strcmp(f, "binary") == 0 ? FDTD_SNAPSHOT_BINARY
                     : std::strcmp(f, "both") == 0 ? FDTD_SNAPSHOT_TEXT_AND_BINARY
                                                   : FDTD_SNAPSHOT_TEXT;
        }
        else if (a == "--timeskip") timeskip = std::strtof(next(), nullptr);
        else if (a == "--kernel") {
            const char *k = next();
            kernel = std::strcmp(k, "two") == 0         ? FDTD_KERNEL_TWO_PASS
                     : std::strcmp(k, "compact") == 0   ? FDTD_KERNEL_COMPACT
                     : std::strcmp(k, "compact16") == 0 ? FDTD_KERNEL_COMPACT_R16
                                                        : FDTD_KERNEL_SINGLE_PASS;
        }
        else if (a == "--device") device = std::atoi(next());
        else if (a == "--voxel-cache") voxel_cache = next();
        else {
            std::fprintf(stderr, "usage: %s [--params P] [--specs P] [--scheme reference|corrected] [--every N] "
                                 "[--fields hx,...] [--format text|binary|both] [--timeskip X] [--kernel single|two|compact|compact16] [--voxel-cache P] [--device N]\n", argv[0]);
            return 2;
        }
    }

    FdtdParams p;
    int st = fdtd_params_read(params_path.c_str(), &p);
    if (st != FDTD_OK)
        return fail(params_path.c_str(), st);
    if (timeskip != 1.0f && (st = fdtd_params_set_timeskip(&p, timeskip)) != FDTD_OK)
        return fail("timeskip", st);
    std::printf("Field size:                 %04dx%04dx%04d\n", p.nx, p.ny, p.nz);
    std::printf("Iterations count:           %d\n", p.iterationsCount);
    std::printf("Input path:                 %s\n", p.inputPath);
    std::printf("Output path:                %s\n", p.outputPath);
    std::printf("dx = %.6e m, dt = %.6e s, sources = %d\n", p.dx, p.dt, p.sourcesCount);

    std::vector<float> specs(4 * FDTD_MAX_CLASSES);
    if ((st = fdtd_read_specs(specs_path.c_str(), specs.data())) != FDTD_OK)
        return fail(specs_path.c_str(), st);
    const size_t n = (size_t)p.nx * p.ny * p.nz;
    std::vector<uint8_t> codes(n);
    auto t0 = std::chrono::steady_clock::now();
    int cached = 0;
    st = voxel_cache.empty() ? fdtd_load_material_codes(&p, p.inputPath, codes.data(), 0)
                             : fdtd_load_material_codes_cached(&p, p.inputPath, voxel_cache.c_str(), codes.data(), 0,
                                                               &cached);
    if (st != FDTD_OK)
        return fail("material slices", st);
    int nclasses = 1;
    for (uint8_t c : codes)
        nclasses = c + 1 > nclasses ? c + 1 : nclasses;
    if ((st = fdtd_setup_sources(&p)) != FDTD_OK)
        return fail("sources", st);

    fdtd_solver_config cfg{};
    cfg.params = &p;
    cfg.material = codes.data();
    cfg.specs = specs.data();
    cfg.nclasses = nclasses;
    cfg.scheme = scheme;
    cfg.kernel = kernel;
    cfg.device = device;
    fdtd_solver *s = nullptr;
    if ((st = fdtd_solver_create(&cfg, &s)) != FDTD_OK)
        return fail("solver", st);
    if (kernel == FDTD_KERNEL_COMPACT || kernel == FDTD_KERNEL_COMPACT_R16)
        mask &= ~(7u << FDTD_FIELD_DX);  // the compact forms store no D
    if (every > 0 && mask) {
        fdtd_snapshot_spec spec{};
        spec.every = every;
        spec.field_mask = mask;
        spec.output_dir = p.outputPath;
        spec.format = format;
        if ((st = fdtd_solver_set_snapshots(s, &spec)) != FDTD_OK)
            return fail("snapshots", st);
    }
    auto t1 = std::chrono::steady_clock::now();
    if ((st = fdtd_solver_run(s, p.iterationsCount)) != FDTD_OK)
        return fail("run", st);
    if ((st = fdtd_solver_flush_snapshots(s)) != FDTD_OK)
        return fail("snapshot output", st);
    if ((st = fdtd_solver_synchronize(s)) != FDTD_OK)
        return fail("run", st);
    auto t2 = std::chrono::steady_clock::now();
    const double setup = std::chrono::duration<double>(t1 - t0).count();
    const double run = std::chrono::duration<double>(t2 - t1).count();
    std::printf("set-up %.3f s%s, %d steps %.3f s (%.3e cell-updates/s including output)\n", setup,
                voxel_cache.empty() ? "" : cached ? " (voxels from cache)" : " (voxel cache written)",
                p.iterationsCount, run, (double)n * p.iterationsCount / run);
    fdtd_solver_destroy(s);
    fdtd_params_free(&p);
    return 0;
}
