// pybind11 module _hoomd_gb300: the host engine classes under the names of the reference's
// C++ classes that the Python layer looks up (hoomd/md/pair/pair.py:126-146,
// hoomd/md/nlist.py:390-397, hoomd/md/integrate.py:287-293).
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <type_traits>
#include <vector>

#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "engine.h"
#include "ensemble.h"
#include "surrogate.h"

namespace py = pybind11;
using namespace gbe;

namespace
{
template<class T> py::array_t<T> make_array(std::vector<size_t> shape)
    {
    return py::array_t<T>(shape);
    }

// Page-locked host blocks for snapshot arrays. A block is handed out wrapped in a capsule that
// owns it; numpy arrays viewing the block keep the capsule alive, and when the last one goes the
// block returns to a small free list (at most POOL_KEEP blocks are kept; more are released).
// Blocks are never shared by two live snapshots. Where page-locked memory cannot be had the
// block is ordinary heap memory.
struct PinnedBlock
    {
    void* ptr = nullptr;
    size_t bytes = 0;
    bool pinned = false;
    };
std::mutex g_pool_mutex;
std::vector<PinnedBlock> g_pool;
constexpr size_t POOL_KEEP = 4;

void release_block(PinnedBlock* b)
    {
    std::unique_ptr<PinnedBlock> own(b);
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (g_pool.size() < POOL_KEEP)
        {
        g_pool.push_back(*b);
        return;
        }
    if (b->pinned)
        cudaFreeHost(b->ptr);
    else
        std::free(b->ptr);
    }

py::capsule pinned_block(size_t bytes)
    {
    PinnedBlock blk;
        {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        // the smallest free block that is large enough
        size_t best = g_pool.size();
        for (size_t k = 0; k < g_pool.size(); k++)
            if (g_pool[k].bytes >= bytes && (best == g_pool.size() || g_pool[k].bytes < g_pool[best].bytes))
                best = k;
        if (best < g_pool.size())
            {
            blk = g_pool[best];
            g_pool.erase(g_pool.begin() + (long)best);
            }
        }
    if (!blk.ptr)
        {
        blk.bytes = std::max<size_t>(bytes, 256);
        blk.pinned = cudaHostAlloc(&blk.ptr, blk.bytes, cudaHostAllocDefault) == cudaSuccess;
        if (!blk.pinned)
            {
            cudaGetLastError();
            blk.ptr = std::malloc(blk.bytes);
            if (!blk.ptr)
                throw std::bad_alloc();
            }
        }
    auto* holder = new PinnedBlock(blk);
    return py::capsule(holder, "gb_snapshot_block",
                       [](PyObject* o) {
                           auto* h = static_cast<PinnedBlock*>(
                               PyCapsule_GetPointer(o, "gb_snapshot_block"));
                           if (h)
                               release_block(h);
                       });
    }

void* pinned_ptr(const py::capsule& c)
    {
    return static_cast<PinnedBlock*>(PyCapsule_GetPointer(c.ptr(), "gb_snapshot_block"))->ptr;
    }

// Per-particle float4 (or 6 x pitch) device array -> numpy in tag order.
py::array_t<double> force_by_tag(PairForce& f, int what)
    {
    ParticleData& pd = *f.pdata;
    const unsigned int N = pd.N;
    std::vector<uint32_t> r = pd.rtag();
    if (what == 2)
        {
        if (!f.virial_valid)
            f.compute(pd.stream, true);
        std::vector<float> h(6 * (size_t)N);
        f.virial.download(h.data(), h.size(), pd.stream);
        cuda_check(cudaStreamSynchronize(pd.stream), "virials");
        auto out = make_array<double>({N, 6});
        auto o = out.mutable_unchecked<2>();
        for (unsigned int t = 0; t < N; t++)
            for (int k = 0; k < 6; k++)
                o(t, k) = h[(size_t)k * N + r[t]];
        return out;
        }
    std::vector<float> h(4 * (size_t)N);
    f.force.download(h.data(), h.size(), pd.stream);
    cuda_check(cudaStreamSynchronize(pd.stream), "forces");
    if (what == 0)
        {
        auto out = make_array<double>({N, 3});
        auto o = out.mutable_unchecked<2>();
        for (unsigned int t = 0; t < N; t++)
            for (int k = 0; k < 3; k++)
                o(t, k) = h[4 * (size_t)r[t] + k];
        return out;
        }
    auto out = make_array<double>({N});
    auto o = out.mutable_unchecked<1>();
    for (unsigned int t = 0; t < N; t++)
        o(t) = h[4 * (size_t)r[t] + 3];
    return out;
    }
// The reference's Python-facing pair force (export_PotentialPair[GPU]<E>,
// hoomd/md/PotentialPair.h:1017-1036): the engine's PairForce plus per-type-pair parameters set
// and read as dicts keyed by type names, r_cut / r_on per type pair, mode by name and the
// tail-correction flag.
struct PyPairForce : PairForce
    {
    PyPairForce(std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl, PairKind k,
                int radial = -1, bool lj_dpd = false)
        : PairForce(std::move(pd), std::move(nl), k), radial_kind(radial), dpd_is_lj(lj_dpd)
        {
        }
    ~PyPairForce()
        {
        if (Py_IsInitialized())
            {
            py::gil_scoped_acquire gil;
            py_params.clear();
            to_bytes = py::object();
            to_dict = py::object();
            }
        }
    int radial_kind;     // the closed form of PairKind::Radial
    bool dpd_is_lj;      // PairKind::DPD: DPDLJ (epsilon, sigma) instead of DPD (A)
    bool tail_correction = false;
    std::map<std::pair<unsigned int, unsigned int>, py::object> py_params; // as given
    py::object to_bytes, to_dict; // PairKind::Plugin: param_type(dict) and param_type::asDict
    };

// parameter names of the radial closed forms, in gb_radial_param.v order (by radial kind)
const std::vector<std::vector<const char*>>& radial_keys()
    {
    static const std::vector<std::vector<const char*>> k = {
        {"epsilon", "sigma"},                       // 0 Gauss
        {"epsilon", "kappa"},                       // 1 Yukawa
        {"D0", "alpha", "r0"},                      // 2 Morse
        {"sigma", "epsilon"},                       // 3 ForceShiftedLJ
        {"epsilon", "sigma", "n", "m"},             // 4 Mie
        {"epsilon", "sigma", "n", "m", "delta"},    // 5 ExpandedMie
        {"sigma", "epsilon", "delta"},              // 6 ExpandedLJ
        {"A", "rho", "C"},                          // 7 Buckingham
        {"sigma", "epsilon"},                       // 8 LJ1208
        {"sigma", "epsilon"},                       // 9 LJ0804
        {"epsilon", "sigma", "r0"},                 // 10 LJGauss
        {"epsilon", "sigma", "delta"},              // 11 ExpandedGaussian
        {"C1", "C2", "eta1", "eta2", "k", "phi"},   // 12 OPP
        {"sigma", "epsilon", "alpha"},              // 13 TWF
        {"A"},                                      // 14 DPDConservative
        {"kappa", "Z", "A", "a1", "a2"},            // 15 DLVO
        {},                                         // 16 Fourier (a, b: three each)
        {"qi", "qj", "aF"},                         // 17 Moliere
        {"qi", "qj", "aF"},                         // 18 ZBL
        {"epsilon", "eps_rf"},                      // 19 ReactionField
        {"kappa"}};                                 // 20 Ewald (+ alpha, default 0)
    return k;
    }

unsigned int type_of(const ParticleData& pd, const py::handle& h)
    {
    if (py::isinstance<py::str>(h))
        {
        const std::string name = h.cast<std::string>();
        for (size_t t = 0; t < pd.type_names.size(); t++)
            if (pd.type_names[t] == name)
                return (unsigned int)t;
        throw py::key_error("unknown particle type " + name);
        }
    const long t = h.cast<long>();
    if (t < 0 || (unsigned long)t >= pd.ntypes)
        throw py::index_error("particle type index out of range");
    return (unsigned int)t;
    }

std::pair<unsigned int, unsigned int> type_pair(const PyPairForce& f, const py::tuple& t)
    {
    if (t.size() != 2)
        throw py::value_error("a type pair is a tuple of two particle types");
    unsigned int a = type_of(*f.pdata, t[0]), b = type_of(*f.pdata, t[1]);
    return {std::min(a, b), std::max(a, b)};
    }

std::vector<double> doubles(const py::handle& h)
    {
    auto a = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(h);
    if (!a)
        throw py::value_error("expected an array of numbers");
    return std::vector<double>(a.data(), a.data() + a.size());
    }

// PotentialPair<E>::setParamsPython: the evaluator's param_type from a dict
void apply_params(PyPairForce& f, unsigned int i, unsigned int j, const py::dict& d)
    {
    auto num = [&](const char* k) {
        if (!d.contains(k))
            throw py::key_error(std::string("missing parameter ") + k);
        return d[k].cast<double>();
    };
    switch (f.kind)
        {
    case PairKind::LJ:
        f.set_params_lj(i, j, num("sigma"), num("epsilon"));
        break;
    case PairKind::Example:
        f.set_params_example(i, j, num("k"), num("sigma"));
        break;
    case PairKind::Table:
        {
        std::vector<double> U = doubles(d["U"]), F = doubles(d["F"]);
        if (U.size() != F.size())
            throw py::value_error("The length of V and F arrays must be equal.");
        if (U.empty())
            throw py::value_error("The length of V and F must not be zero.");
        f.set_params_table(i, j, num("r_min"), U, F);
        break;
        }
    case PairKind::DPD:
        if (f.dpd_is_lj)
            f.set_params_dpd(i, j, true, num("epsilon"), num("sigma"), num("gamma"));
        else
            f.set_params_dpd(i, j, false, num("A"), 0.0, num("gamma"));
        break;
    case PairKind::Radial:
        {
        std::vector<double> v;
        if (f.radial_kind == 16)
            {
            std::vector<double> a = doubles(d["a"]), b = doubles(d["b"]);
            if (a.size() != 3 || b.size() != 3)
                throw py::value_error("Fourier: a and b are three coefficients each");
            v = {a[0], a[1], a[2], b[0], b[1], b[2]};
            }
        else
            {
            for (const char* k : radial_keys().at(f.radial_kind))
                v.push_back(num(k));
            if (f.radial_kind == 20)
                v.push_back(d.contains("alpha") ? d["alpha"].cast<double>() : 0.0);
            }
        f.set_params_radial(i, j, (unsigned int)f.radial_kind, v);
        break;
        }
    case PairKind::Plugin:
        {
        const std::string rec = py::bytes(f.to_bytes(d));
        f.set_params_plugin(i, j, rec.data(), rec.size());
        break;
        }
    default:
        throw py::type_error("this pair force takes no per-type-pair parameters");
        }
    f.py_params[{i, j}] = py::dict(d);
    }

py::dict read_params(PyPairForce& f, unsigned int i, unsigned int j)
    {
    if (f.kind == PairKind::Plugin)
        {
        const size_t b = f.plugin->param_size;
        const unsigned char* r = f.plugin_params.data() + (size_t)(i * f.ntypes + j) * b;
        return f.to_dict(py::bytes(reinterpret_cast<const char*>(r), b));
        }
    auto it = f.py_params.find({i, j});
    if (it == f.py_params.end())
        throw py::key_error("parameters of this type pair are not set");
    return py::dict(it->second);
    }

std::shared_ptr<PyPairForce> make_pair_force(std::shared_ptr<ParticleData> pd,
                                             std::shared_ptr<NeighborList> nl, PairKind k,
                                             int radial = -1, bool lj_dpd = false)
    {
    auto f = std::make_shared<PyPairForce>(std::move(pd), std::move(nl), k, radial, lj_dpd);
    f->uses_charge = k == PairKind::Plugin;
    return f;
    }

const char* mode_name(int m)
    {
    return m == 1 ? "shift" : (m == 2 ? "xplor" : "none");
    }
} // namespace

PYBIND11_MODULE(_hoomd_gb300, m)
    {
    m.doc() = "GB300-native short-range MD engine (host classes over the C ABI)";
    m.def("version", []() { return gb_version(); });

    py::class_<ParticleData, std::shared_ptr<ParticleData>>(m, "ParticleData")
        .def(py::init<unsigned int, unsigned int, unsigned int, std::vector<double>,
                      std::vector<int>>())
        .def("setParticles",
             [](ParticleData& pd, py::array_t<double, py::array::c_style | py::array::forcecast> pos,
                py::array_t<double, py::array::c_style | py::array::forcecast> vel,
                py::array_t<double, py::array::c_style | py::array::forcecast> mass,
                py::array_t<uint32_t, py::array::c_style | py::array::forcecast> typeid_,
                py::array_t<int32_t, py::array::c_style | py::array::forcecast> image,
                py::object charge) {
                 const size_t N = pd.N;
                 if ((size_t)pos.size() != 3 * N || (size_t)vel.size() != 3 * N
                     || (size_t)mass.size() != N || (size_t)typeid_.size() != N
                     || (size_t)image.size() != 3 * N)
                     throw std::invalid_argument("particle array sizes do not match N");
                 if (charge.is_none())
                     {
                     pd.set_particles(pos.data(), vel.data(), mass.data(), typeid_.data(),
                                      image.data(), nullptr);
                     return;
                     }
                 auto q = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(
                     charge);
                 if (!q || (size_t)q.size() != N)
                     throw std::invalid_argument("charge array size does not match N");
                 pd.set_particles(pos.data(), vel.data(), mass.data(), typeid_.data(),
                                  image.data(), q.data());
             },
             py::arg("pos"), py::arg("vel"), py::arg("mass"), py::arg("typeid"),
             py::arg("image"), py::arg("charge") = py::none())
        .def("setCharges",
             [](ParticleData& pd, py::array_t<double, py::array::c_style | py::array::forcecast> q) {
                 if ((size_t)q.size() != pd.N)
                     throw std::invalid_argument("charge array size does not match N");
                 pd.set_charges(q.data());
             })
        .def("getParticles",
             [](ParticleData& pd) {
                 const size_t N = pd.N;
                 // the five arrays share one page-locked block (the device writes them at full
                 // link speed, no page faults), recycled when the arrays are released
                 auto up = [](size_t b) { return (b + 255) / 256 * 256; };
                 const size_t o_vel = up(24 * N), o_mass = o_vel + up(24 * N),
                              o_tid = o_mass + up(8 * N), o_img = o_tid + up(4 * N),
                              total = o_img + up(12 * N);
                 py::capsule owner = pinned_block(total);
                 char* base = static_cast<char*>(pinned_ptr(owner));
                 auto view = [&](auto* ptr, std::vector<size_t> shape) {
                     using T = std::remove_pointer_t<decltype(ptr)>;
                     return py::array_t<T>(shape, ptr, owner);
                 };
                 auto pos = view(reinterpret_cast<double*>(base), {N, 3});
                 auto vel = view(reinterpret_cast<double*>(base + o_vel), {N, 3});
                 auto mass = view(reinterpret_cast<double*>(base + o_mass), {N});
                 auto tid = view(reinterpret_cast<uint32_t*>(base + o_tid), {N});
                 auto img = view(reinterpret_cast<int32_t*>(base + o_img), {N, 3});
                 pd.get_particles(pos.mutable_data(), vel.mutable_data(), mass.mutable_data(),
                                  tid.mutable_data(), img.mutable_data());
                 py::dict d;
                 d["position"] = pos;
                 d["velocity"] = vel;
                 d["mass"] = mass;
                 d["typeid"] = tid;
                 d["image"] = img;
                 return d;
             })
        .def("thermalize", &ParticleData::thermalize)
        .def_readwrite("seed", &ParticleData::seed)
        .def_readwrite("timestep", &ParticleData::timestep)
        .def_readonly("N", &ParticleData::N)
        .def_readonly("ntypes", &ParticleData::ntypes)
        .def_readonly("ndim", &ParticleData::ndim)
        .def_readonly("sort_generation", &ParticleData::sort_generation)
        .def_readwrite("types", &ParticleData::type_names)
        .def("getBox",
             [](ParticleData& pd) {
                 return std::vector<double>(pd.box6, pd.box6 + 6);
             });

    py::class_<NeighborList, std::shared_ptr<NeighborList>>(m, "NeighborListGPUBinned")
        .def(py::init<std::shared_ptr<ParticleData>, double>())
        .def("setRCut", &NeighborList::set_r_cut)
        .def("setExclusions",
             [](NeighborList& n, py::array_t<uint32_t, py::array::c_style | py::array::forcecast> p) {
                 n.set_exclusions(std::vector<uint32_t>(p.data(), p.data() + p.size()));
                 n.dirty = true;
             })
        .def_property_readonly("ex_pitch", [](NeighborList& n) { return n.ex_pitch; })
        .def_property(
            "deterministic", [](NeighborList& n) { return n.deterministic; },
            [](NeighborList& n, bool v) {
                n.deterministic = v;
                n.dirty = true;
            })
        .def_property(
            "r_buff", [](NeighborList& n) { return n.r_buff; },
            [](NeighborList& n, double v) {
                if (v < 0)
                    throw std::invalid_argument("Requested buffer radius is less than zero.");
                n.r_buff = (float)v;
                n.dirty = true;
            })
        .def_readwrite("check_dist", &NeighborList::check_dist)
        .def_readwrite("rebuild_check_delay", &NeighborList::rebuild_check_delay)
        .def("getDim", &NeighborList::dims)
        .def("getAutotunerParameters",
             [](NeighborList& n) {
                 py::dict d;
                 d["nlist"] = py::make_tuple(n.kp_block ? n.kp_block : 128u,
                                             n.kp_tpp ? n.kp_tpp : 32u);
                 return d;
             })
        .def("setAutotunerParameters",
             [](NeighborList& n, py::dict d) {
                 for (auto kv : d)
                     {
                     if (py::str(kv.first).cast<std::string>() != "nlist")
                         throw py::key_error("no kernel " + py::str(kv.first).cast<std::string>());
                     auto t = kv.second.cast<std::vector<unsigned int>>();
                     if (t.size() != 2 || (t[0] != 32 && t[0] != 64 && t[0] != 128)
                         || (t[1] != 1 && t[1] != 32))
                         throw py::value_error(
                             "nlist: (block size 32, 64 or 128, threads per particle 1 or 32)");
                     n.kp_block = t[0];
                     n.kp_tpp = t[1];
                     }
                 n.tune_requested = false;
             })
        .def("isAutotuningComplete", [](NeighborList& n) { return !n.tune_requested; })
        .def("startAutotuning", [](NeighborList& n) { n.tune_requested = true; })
        .def("getNmax", [](NeighborList& n) { return n.Nmax_cell; })
        .def("getNmaxPerType", [](NeighborList& n) { return n.Nmax; })
        .def("getRList", [](NeighborList& n) { return n.r_listsq; })
        .def("getPairList",
             [](NeighborList& n, bool full, bool local) {
                 std::vector<uint32_t> v = n.pair_list(full, local);
                 auto out = make_array<uint32_t>({v.size() / 2, 2});
                 std::copy(v.begin(), v.end(), out.mutable_data());
                 return out;
             },
             py::arg("full"), py::arg("local") = false)
        .def("getNNeigh",
             [](NeighborList& n) {
                 ParticleData& pd = *n.pdata;
                 std::vector<uint32_t> h(pd.N);
                 n.n_neigh.download(h.data(), pd.N, pd.stream);
                 std::vector<uint32_t> r = pd.rtag();
                 auto out = make_array<uint32_t>({(size_t)pd.N});
                 auto o = out.mutable_unchecked<1>();
                 for (unsigned int t = 0; t < pd.N; t++)
                     o(t) = h[r[t]];
                 return out;
             })
        .def("buildNow", &NeighborList::build_sync)
        .def_readonly("alloc_generation", &NeighborList::alloc_generation)
        .def("setStartCapacity",
             [](NeighborList& n, unsigned int cell, std::vector<uint32_t> per_type) {
                 if (per_type.size() != n.pdata->ntypes)
                     throw std::invalid_argument("one capacity per particle type");
                 n.Nmax_cell = cell;
                 n.Nmax = per_type;
                 n.capacity_fixed = true;
                 n.allocated = false;
                 n.dirty = true;
             });

    py::enum_<PairKind>(m, "PairKind")
        .value("LJ", PairKind::LJ)
        .value("Table", PairKind::Table)
        .value("Example", PairKind::Example)
        .value("MLP", PairKind::MLP)
        .value("Radial", PairKind::Radial)
        .value("DPD", PairKind::DPD)
        .value("Plugin", PairKind::Plugin);

    py::class_<PairForce, std::shared_ptr<PairForce>>(m, "PotentialPairGPU")
        .def(py::init([](std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl,
                         PairKind k) -> std::shared_ptr<PairForce> {
            return make_pair_force(std::move(pd), std::move(nl), k);
        }))
        .def("setParamsLJ", &PairForce::set_params_lj)
        .def("setParamsExample", &PairForce::set_params_example)
        // Autotuner interface (hoomd/Autotuner.h, AutotunedObject in hoomd/operation.py)
        .def("getAutotunerParameters",
             [](PairForce& f) {
                 // the values in use: the set ones, else the kernel's defaults
                 const unsigned int N = f.pdata->N;
                 const unsigned int tpp
                     = f.kp_tpp ? f.kp_tpp : (N <= 16384 ? 8u : (N <= 65536 ? 4u : 1u));
                 py::dict d;
                 d["pair"] = py::make_tuple(f.kp_block ? f.kp_block : 256u, tpp);
                 return d;
             })
        .def("setAutotunerParameters",
             [](PairForce& f, py::dict d) {
                 for (auto kv : d)
                     {
                     if (py::str(kv.first).cast<std::string>() != "pair")
                         throw py::key_error("no kernel " + py::str(kv.first).cast<std::string>());
                     auto t = kv.second.cast<std::vector<unsigned int>>();
                     if (t.size() != 2 || (t[0] != 128 && t[0] != 256)
                         || (t[1] != 1 && t[1] != 4 && t[1] != 8))
                         throw py::value_error("pair: (block size 128 or 256, threads per "
                                               "particle 1, 4 or 8)");
                     f.kp_block = t[0];
                     f.kp_tpp = t[1];
                     }
                 f.tune_requested = false;
             })
        .def("isAutotuningComplete", [](PairForce& f) { return !f.tune_requested; })
        .def("startAutotuning", [](PairForce& f) { f.tune_requested = true; })
        .def("setParamsTable", &PairForce::set_params_table)
        .def("setParamsRadial", &PairForce::set_params_radial)
        .def("setParamsDPD", &PairForce::set_params_dpd)
        .def_readwrite("dpdKT", &PairForce::dpd_kT)
        .def_readwrite("useCharge", &PairForce::uses_charge)
        .def("setTailCorrection",
             [](PairForce& f, double energy, double virial) {
                 f.tail_energy = energy;
                 f.tail_virial = virial;
             })
        .def("tailEnergy", [](PairForce& f) { return f.tail_energy / f.box_volume(); })
        .def("tailVirial", [](PairForce& f) { return f.tail_virial / f.box_volume(); })
        .def("setRCut", &PairForce::set_r_cut)
        .def("setROn", &PairForce::set_r_on)
        .def("setSurrogate", [](PairForce& f, std::shared_ptr<MlpSurrogate> m) { f.mlp = m; })
        .def_property(
            "mode", [](PairForce& f) { return std::string(mode_name(f.shift_mode)); },
            [](PairForce& f, py::object v) {
                int mv = -1;
                if (py::isinstance<py::str>(v))
                    {
                    const std::string s = v.cast<std::string>();
                    mv = s == "none" ? 0 : (s == "shift" ? 1 : (s == "xplor" ? 2 : -1));
                    }
                else
                    mv = v.cast<int>();
                if (mv < 0 || mv > 2)
                    throw std::invalid_argument("mode must be 'none', 'shift' or 'xplor'");
                f.shift_mode = mv;
                f.params_dirty = true;
            })
        .def("compute", &PairForce::compute_standalone)
        .def("computeEnergyBetweenSets",
             [](PairForce& f, py::array_t<int64_t, py::array::c_style | py::array::forcecast> a,
                py::array_t<int64_t, py::array::c_style | py::array::forcecast> b) {
                 auto conv = [](const py::array_t<int64_t, py::array::c_style
                                                               | py::array::forcecast>& x) {
                     std::vector<uint32_t> v((size_t)x.size());
                     for (size_t k = 0; k < v.size(); k++)
                         {
                         if (x.data()[k] < 0)
                             throw std::invalid_argument("compute_energy: negative tag");
                         v[k] = (uint32_t)x.data()[k];
                         }
                     return v;
                 };
                 return f.energy_between_sets(conv(a), conv(b));
             })
        .def("getForces", [](PairForce& f) { return force_by_tag(f, 0); })
        .def("getEnergies", [](PairForce& f) { return force_by_tag(f, 1); })
        .def("energySum", &PairForce::energy_sum)
        .def("getVirials", [](PairForce& f) { return force_by_tag(f, 2); });

    // one class for every evaluator; the reference's per-evaluator class names
    // (PotentialPair<Name>GPU, hoomd/md/pair/pair.py _cpp_class_name + "GPU") construct it
    py::class_<PyPairForce, PairForce, std::shared_ptr<PyPairForce>>(m, "PotentialPairEvaluatorGPU")
        .def("setParams",
             [](PyPairForce& f, py::tuple typ, py::dict d) {
                 auto ij = type_pair(f, typ);
                 apply_params(f, ij.first, ij.second, d);
             })
        .def("getParams",
             [](PyPairForce& f, py::tuple typ) {
                 auto ij = type_pair(f, typ);
                 return read_params(f, ij.first, ij.second);
             })
        .def("setRCut",
             [](PyPairForce& f, py::tuple typ, double r) {
                 auto ij = type_pair(f, typ);
                 f.set_r_cut(ij.first, ij.second, r);
             })
        .def("getRCut",
             [](PyPairForce& f, py::tuple typ) {
                 auto ij = type_pair(f, typ);
                 return (double)f.r_cut[ij.first * f.ntypes + ij.second];
             })
        .def("setROn",
             [](PyPairForce& f, py::tuple typ, double r) {
                 auto ij = type_pair(f, typ);
                 f.set_r_on(ij.first, ij.second, r);
             })
        .def("getROn",
             [](PyPairForce& f, py::tuple typ) {
                 auto ij = type_pair(f, typ);
                 return (double)f.r_on[ij.first * f.ntypes + ij.second];
             })
        .def_readwrite("tail_correction", &PyPairForce::tail_correction)
        .def_property_readonly("evaluator_name", [](PyPairForce& f) {
            return f.kind == PairKind::Plugin && f.plugin && f.plugin->name
                       ? std::string(f.plugin->name)
                       : std::string();
        });
    {
    struct Named
        {
        const char* name;
        PairKind kind;
        int radial;
        bool lj_dpd;
        };
    static const Named named[] = {
        {"PotentialPairLJGPU", PairKind::LJ, -1, false},
        {"PotentialPairTableGPU", PairKind::Table, -1, false},
        {"PotentialPairExampleGPU", PairKind::Example, -1, false},
        {"PotentialPairGaussGPU", PairKind::Radial, 0, false},
        {"PotentialPairYukawaGPU", PairKind::Radial, 1, false},
        {"PotentialPairMorseGPU", PairKind::Radial, 2, false},
        {"PotentialPairForceShiftedLJGPU", PairKind::Radial, 3, false},
        {"PotentialPairMieGPU", PairKind::Radial, 4, false},
        {"PotentialPairExpandedMieGPU", PairKind::Radial, 5, false},
        {"PotentialPairExpandedLJGPU", PairKind::Radial, 6, false},
        {"PotentialPairBuckinghamGPU", PairKind::Radial, 7, false},
        {"PotentialPairLJ1208GPU", PairKind::Radial, 8, false},
        {"PotentialPairLJ0804GPU", PairKind::Radial, 9, false},
        {"PotentialPairLJGaussGPU", PairKind::Radial, 10, false},
        {"PotentialPairExpandedGaussianGPU", PairKind::Radial, 11, false},
        {"PotentialPairOPPGPU", PairKind::Radial, 12, false},
        {"PotentialPairTWFGPU", PairKind::Radial, 13, false},
        {"PotentialPairConservativeDPDGPU", PairKind::Radial, 14, false},
        {"PotentialPairDLVOGPU", PairKind::Radial, 15, false},
        {"PotentialPairFourierGPU", PairKind::Radial, 16, false},
        {"PotentialPairMoliereGPU", PairKind::Radial, 17, false},
        {"PotentialPairZBLGPU", PairKind::Radial, 18, false},
        {"PotentialPairReactionFieldGPU", PairKind::Radial, 19, false},
        {"PotentialPairEwaldGPU", PairKind::Radial, 20, false},
        {"PotentialPairDPDThermoDPDGPU", PairKind::DPD, -1, false},
        {"PotentialPairDPDThermoLJGPU", PairKind::DPD, -1, true}};
    for (const Named& n : named)
        {
        const Named c = n;
        m.def(c.name,
              [c](std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl) {
                  return make_pair_force(std::move(pd), std::move(nl), c.kind, c.radial,
                                         c.lj_dpd);
              },
              py::arg("sysdef"), py::arg("nlist"));
        }
    }
    // a plugin evaluator's pair force: built by the plugin module's export_PotentialPairGPU<E>
    // (include/hoomd/md/PotentialPairGPU.h) from its gb_pair_plugin record and its param_type
    // conversions
    m.def("PotentialPairPluginGPU",
          [](std::shared_ptr<ParticleData> pd, std::shared_ptr<NeighborList> nl, py::capsule rec,
             py::object to_bytes, py::object to_dict) {
              if (std::string(rec.name() ? rec.name() : "") != "gb_pair_plugin")
                  throw py::type_error("expected a gb_pair_plugin capsule");
              const auto* r = static_cast<const gb_pair_plugin*>(rec.get_pointer());
              if (!r || r->abi != GB_PAIR_PLUGIN_ABI || !r->call || r->param_size == 0)
                  throw py::value_error("pair plugin record of an incompatible ABI version");
              auto f = make_pair_force(std::move(pd), std::move(nl), PairKind::Plugin);
              f->plugin = r;
              f->plugin_params.assign((size_t)f->ntypes * f->ntypes * r->param_size, 0);
              f->to_bytes = std::move(to_bytes);
              f->to_dict = std::move(to_dict);
              return f;
          });

    py::class_<Integrator, std::shared_ptr<Integrator>>(m, "IntegratorTwoStep")
        .def(py::init<std::shared_ptr<ParticleData>, std::shared_ptr<NeighborList>, double>())
        .def("addForce", &Integrator::add_force)
        .def("lastTuning",
             [](Integrator& in) {
                 py::list out;
                 for (auto& t : in.last_tuning)
                     out.append(py::make_tuple(t.kernel, t.block, t.tpp, t.ms));
                 return out;
             })
        .def("setBussi", &Integrator::set_thermostat_bussi)
        .def("setNoThermostat", &Integrator::set_thermostat_none)
        .def("setLangevin", &Integrator::set_langevin)
        .def("setBrownian", &Integrator::set_brownian)
        .def("setMaxDisplacement", &Integrator::set_max_displacement)
        .def("setNPT", &Integrator::set_npt)
        .def("getBarostatDOF", &Integrator::barostat_dof)
        .def("setBarostatDOF", &Integrator::set_barostat_dof)
        .def("barostatEnergy", &Integrator::barostat_energy)
        .def("thermoTensor", &Integrator::thermo_tensor)
        .def("setBerendsen", &Integrator::set_thermostat_berendsen)
        .def("setMTTK", &Integrator::set_thermostat_mttk)
        .def("getMTTKState", &Integrator::mttk_state)
        .def("setMTTKState", &Integrator::set_mttk_state)
        .def("thermalizeMTTK", &Integrator::thermalize_mttk)
        .def("mttkEnergy", &Integrator::mttk_energy)
        .def_property_readonly("reservoir_energy", &Integrator::reservoir_energy)
        .def("setSorter", &Integrator::set_sorter)
        .def("setChunk", &Integrator::set_chunk)
        .def_readwrite("use_graph", &Integrator::use_graph)
        .def_readwrite("notice_level", &Integrator::notice_level)
        .def_property(
            "conditional_build", [](const Integrator& in) { return in.use_conditional_build; },
            [](Integrator& in, bool v) {
                in.use_conditional_build = v;
                in.drop_graphs();
            })
        .def_readwrite("compute_virial", &Integrator::compute_virial)
        .def_readonly("n_rollbacks", &Integrator::n_rollbacks)
        .def("graphCount", &Integrator::graph_count)
        .def("resetBuildStats", &Integrator::reset_build_stats)
        .def("graphGeneration", &Integrator::graph_generation)
        .def_readonly("steps_run", &Integrator::steps_run)
        .def_readonly("launch_count", &Integrator::launch_count)
        .def("timePhases", &Integrator::time_phases)
        .def("streamHandle", &Integrator::stream_handle)
        .def("sumNNeigh", &Integrator::sum_n_neigh)
        .def_property(
            "dt", [](Integrator& i) { return i.dt; },
            [](Integrator& i, double v) {
                i.dt = v;
                i.prepared = false;
                i.drop_graphs(); // the captured steps hold the time step
            })
        .def("prepRun", &Integrator::prepare, py::arg("keep_graphs") = false)
        .def("run", &Integrator::run, py::call_guard<py::gil_scoped_release>())
        .def("thermo", &Integrator::thermo)
        .def("dof", &Integrator::dof)
        .def("status",
             [](Integrator& i) {
                 DevStatus st = i.read_status();
                 py::dict d;
                 d["timestep"] = st.timestep;
                 d["n_builds"] = st.n_builds;
                 d["shortest_rebuild"] = st.build_steps[1];
                 d["last_update"] = st.build_steps[0];
                 d["dangerous_builds"] = st.n_dangerous;
                 d["factor"] = st.factor;
                 d["kinetic_energy"] = st.thermo[0];
                 d["potential_energy"] = st.thermo[1];
                 return d;
             })
        .def("synchronize",
             [](Integrator& i) { cuda_check(cudaStreamSynchronize(i.pdata->stream), "sync"); });

    using farr = py::array_t<float, py::array::c_style | py::array::forcecast>;
    using uarr = py::array_t<uint32_t, py::array::c_style | py::array::forcecast>;
    auto fvec = [](const farr& a) { return std::vector<float>(a.data(), a.data() + a.size()); };
    auto uvec = [](const uarr& a) { return std::vector<uint32_t>(a.data(), a.data() + a.size()); };
    py::class_<MlpSurrogate, std::shared_ptr<MlpSurrogate>>(m, "MlpSurrogate")
        .def(py::init<unsigned int, double, double, uint64_t>())
        .def_property_readonly("n_pairs", &MlpSurrogate::n_pairs)
        .def_readonly("ntypes", &MlpSurrogate::ntypes)
        .def_readonly("r_min", &MlpSurrogate::r_min)
        .def_readonly("r_cut", &MlpSurrogate::r_cut)
        .def_readwrite("act_split", &MlpSurrogate::act_split)
        .def_property(
            "tensor_kernel",
            [](const MlpSurrogate& s) { return std::string(s.mma_sync ? "mma.sync" : "tcgen05"); },
            [](MlpSurrogate& s, const std::string& k) {
                if (k != "tcgen05" && k != "mma.sync")
                    throw py::value_error("tensor_kernel: 'tcgen05' or 'mma.sync'");
                s.mma_sync = k == "mma.sync" ? 1 : 0;
            })
        .def_readonly("train_steps", &MlpSurrogate::train_steps)
        .def_readonly("train_ms", &MlpSurrogate::train_ms)
        .def("setParams", [fvec](MlpSurrogate& s, farr th) { s.set_params(fvec(th)); })
        .def("getParams",
             [](MlpSurrogate& s) {
                 std::vector<float> v = s.params();
                 auto out = make_array<float>({v.size()});
                 std::copy(v.begin(), v.end(), out.mutable_data());
                 return out;
             })
        .def("setSamples",
             [fvec, uvec](MlpSurrogate& s, uarr pair, farr r, farr U, farr F) {
                 s.set_samples(uvec(pair), fvec(r), fvec(U), fvec(F));
             })
        .def("train", &MlpSurrogate::train, py::call_guard<py::gil_scoped_release>())
        .def("loss", &MlpSurrogate::loss)
        .def("eval",
             [fvec, uvec](MlpSurrogate& s, uarr pair, farr r) {
                 std::vector<float> U, dU;
                 s.eval(uvec(pair), fvec(r), U, dU);
                 auto a = make_array<float>({U.size()});
                 auto b = make_array<float>({dU.size()});
                 std::copy(U.begin(), U.end(), a.mutable_data());
                 std::copy(dU.begin(), dU.end(), b.mutable_data());
                 return py::make_tuple(a, b);
             });

    using darr = py::array_t<double, py::array::c_style | py::array::forcecast>;
    py::class_<ReplicaEnsemble, std::shared_ptr<ReplicaEnsemble>>(m, "ReplicaEnsembleGPU")
        .def(py::init<double, double, double, double, double, int>())
        .def("addReplica",
             [](ReplicaEnsemble& e, darr pos, darr vel, darr mass,
                py::array_t<int32_t, py::array::c_style | py::array::forcecast> image, darr L,
                darr tilt, bool bussi, double kT, double tau, uint32_t seed, uint64_t timestep) {
                 const size_t N = (size_t)mass.size();
                 if ((size_t)pos.size() != 3 * N || (size_t)vel.size() != 3 * N
                     || (size_t)image.size() != 3 * N || L.size() != 3 || tilt.size() != 3)
                     throw std::invalid_argument("replica array sizes do not match N");
                 return e.add((unsigned int)N, pos.data(), vel.data(), mass.data(), image.data(),
                              L.data(), tilt.data(), bussi, kT, tau, seed, timestep);
             })
        .def("run", &ReplicaEnsemble::run, py::call_guard<py::gil_scoped_release>())
        .def("autotune",
             [](ReplicaEnsemble& e, uint32_t steps, uint32_t repeats) {
                 py::list out;
                 for (const TuneResult& t : e.autotune(steps, repeats))
                     out.append(py::make_tuple(t.block_size, t.grid_size, t.ms_per_step));
                 return out;
             })
        .def("setLaunch", &ReplicaEnsemble::set_launch)
        .def("setStartCapacity", &ReplicaEnsemble::set_start_capacity)
        .def("setStencil", &ReplicaEnsemble::set_stencil)
        .def("getParticles",
             [](ReplicaEnsemble& e, uint32_t r) {
                 const size_t N = e.record(r).N;
                 auto pos = make_array<double>({N, 3});
                 auto vel = make_array<double>({N, 4});
                 auto img = make_array<int32_t>({N, 3});
                 auto frc = make_array<double>({N, 4});
                 e.get_particles(r, pos.mutable_data(), vel.mutable_data(), img.mutable_data(),
                                 frc.mutable_data());
                 py::dict d;
                 d["position"] = pos;
                 d["velocity"] = vel;
                 d["image"] = img;
                 d["force"] = frc;
                 return d;
             })
        .def("neighborCounts", &ReplicaEnsemble::neighbor_counts)
        .def("phaseClocks", &ReplicaEnsemble::phase_clocks)
        .def("neighborList",
             [](ReplicaEnsemble& e, uint32_t r) {
                 std::vector<uint32_t> v = e.neighbor_list(r);
                 const gb_replica rec = e.record(r);
                 auto out = make_array<int64_t>({(size_t)rec.N, (size_t)rec.Nmax});
                 int64_t* o = out.mutable_data();
                 for (size_t k = 0; k < v.size(); k++)
                     o[k] = v[k] == 0xffffffffu ? -1 : (int64_t)v[k];
                 return out;
             })
        .def("record",
             [](ReplicaEnsemble& e, uint32_t r) {
                 const gb_replica x = e.record(r);
                 py::dict d;
                 d["N"] = x.N;
                 d["timestep"] = x.timestep;
                 d["kinetic_energy"] = x.ke;
                 d["potential_energy"] = x.pe;
                 d["factor"] = x.factor;
                 d["n_builds"] = x.n_builds;
                 d["Nmax"] = x.Nmax;
                 d["dim"] = std::vector<uint32_t>(x.dim, x.dim + 3);
                 d["stencil"] = x.stencil;
                 d["dof"] = x.dof;
                 d["kT"] = x.kT;
                 d["box"] = std::vector<float>(x.box.L, x.box.L + 3);
                 d["prepared"] = x.prepared;
                 return d;
             })
        .def_property_readonly("count", &ReplicaEnsemble::count)
        .def_property_readonly("total_particles", &ReplicaEnsemble::total_particles)
        .def_readonly("block_size", &ReplicaEnsemble::block_size)
        .def_readonly("grid_size", &ReplicaEnsemble::grid_size)
        .def_readonly("launch_count", &ReplicaEnsemble::launch_count)
        .def_readonly("n_regrowths", &ReplicaEnsemble::n_regrowths)
        .def_readonly("last_run_ms", &ReplicaEnsemble::last_run_ms)
        .def_readwrite("use_graph", &ReplicaEnsemble::use_graph)
        .def("streamHandle", &ReplicaEnsemble::stream_handle);
    }
