// Drives nblib_gb300::ForceCalculator the way nblib's integration tests drive
// nblib::ForceCalculator (api/nblib/tests/nbnxmsetup.cpp, integrator.cpp): build
// a Topology and SimulationState, construct the calculator, compute forces,
// update the pair list and compute again.  Inputs and outputs are little-endian
// binary files written and read by tests/test_nblib_adapter.py.
//
// input : int32 n, ntypes, mode (0 per-type C6/C12 geometric, 1 explicit table,
//         2 per-type C6/C12 Lorentz-Berthelot, other: that CombinationRule
//         value), coulomb, energy;
//         float32 rc, rlist, box[3]; float32 x[3n], q[n]; int32 type[n];
//         float32 params (mode 1: 2*nt*nt, else c6[nt], c12[nt]);
//         int32 excl_index[n+1], excl_list[excl_index[n]]
// output: int32 outcome (0 ok, 1 InputException, 2 GpuException), int32 code,
//         int32 size_check (1 when a wrong-size force buffer raised InputException);
//         float32 f[3n], f_after_update[3n]; float64 energies[2], virial[9];
//         then the message of a failure as text
#include <cstdint>
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "nblib_gb300.hpp"

using namespace nblib_gb300;

namespace
{
template<typename T>
std::vector<T> read_vec(std::FILE* f, std::size_t n)
{
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != n)
    {
        throw std::runtime_error("short input file");
    }
    return v;
}
template<typename T>
void write_vec(std::FILE* f, const T* p, std::size_t n)
{
    std::fwrite(p, sizeof(T), n, f);
}
} // namespace

int main(int argc, char** argv)
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    std::FILE* in = std::fopen(argv[1], "rb");
    if (!in)
    {
        return 2;
    }
    const auto hdr   = read_vec<int32_t>(in, 5);
    const int  n     = hdr[0], nt = hdr[1], mode = hdr[2], coulomb = hdr[3], energy = hdr[4];
    const auto rr    = read_vec<float>(in, 5);
    const auto xs    = read_vec<float>(in, 3 * (std::size_t)n);
    const auto q     = read_vec<float>(in, n);
    const auto types = read_vec<int32_t>(in, n);
    const auto par   = read_vec<float>(in, mode == 1 ? 2 * (std::size_t)nt * nt : 2 * (std::size_t)nt);
    const auto ei    = read_vec<int32_t>(in, (std::size_t)n + 1);
    const auto el    = read_vec<int32_t>(in, ei[n]);
    std::fclose(in);

    std::vector<std::vector<int>> excl(n);
    for (int i = 0; i < n; i++)
    {
        excl[i].assign(el.begin() + ei[i], el.begin() + ei[i + 1]);
    }
    std::vector<Vec3> x(n), f(n), f2(n);
    for (int i = 0; i < n; i++)
    {
        x[i] = { xs[3 * i], xs[3 * i + 1], xs[3 * i + 2] };
    }

    int32_t     outcome = 0, code = 0, size_check = 0;
    std::string message;
    std::array<double, 2> e{};
    std::array<double, 9> vir{};
    try
    {
        std::vector<int> typeIds(types.begin(), types.end());
        std::vector<real> charges(q.begin(), q.end());
        Topology topo = (mode == 1)
                                ? Topology(typeIds, charges, nt, std::vector<real>(par.begin(), par.end()), excl)
                                : Topology(typeIds, charges, std::vector<real>(par.begin(), par.begin() + nt),
                                           std::vector<real>(par.begin() + nt, par.end()),
                                           mode == 0   ? CombinationRule::Geometric
                                           : mode == 2 ? CombinationRule::LorentzBerthelot
                                                       : static_cast<CombinationRule>(mode),
                                           excl);
        SimulationState state(x, std::vector<Vec3>(n), std::vector<Vec3>(n), Box(rr[2], rr[3], rr[4]), topo);
        NBKernelOptions opts;
        opts.coulombType            = static_cast<CoulombType>(coulomb);
        opts.rcoulomb               = rr[0];
        opts.pairlistCutoff         = rr[1];
        opts.computeVirialAndEnergy = energy != 0;
        ForceCalculator calc(state, opts);
        calc.compute(state.coordinates(), f);
        e   = calc.energies();
        vir = calc.virial();
        // a force buffer of the wrong size is an input error, as in nblib
        try
        {
            std::vector<Vec3> small(n > 0 ? n - 1 : 0);
            calc.compute(state.coordinates(), small);
        }
        catch (const InputException&)
        {
            size_check = 1;
        }
        std::vector<int> info(n, 0);
        calc.updatePairList(info, state.coordinates(), state.box());
        calc.compute(state.coordinates(), f2);
    }
    catch (const InputException& ex)
    {
        outcome = 1;
        message = ex.what();
    }
    catch (const GpuException& ex)
    {
        outcome = 2;
        code    = ex.status();
        message = ex.what();
    }

    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out)
    {
        return 2;
    }
    write_vec(out, &outcome, 1);
    write_vec(out, &code, 1);
    write_vec(out, &size_check, 1);
    write_vec(out, f.data()->data(), 3 * (std::size_t)n);
    write_vec(out, f2.data()->data(), 3 * (std::size_t)n);
    write_vec(out, e.data(), 2);
    write_vec(out, vir.data(), 9);
    std::fwrite(message.data(), 1, message.size(), out);
    std::fclose(out);
    return 0;
}
