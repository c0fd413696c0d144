// pybind11 module _hoomd_gb300: the host engine classes under the names of the reference's
// C++ classes that the Python layer looks up (hoomd/md/pair/pair.py:126-146,
// hoomd/md/nlist.py:390-397, hoomd/md/integrate.py:287-293).
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
                 auto pos = make_array<double>({N, 3});
                 auto vel = make_array<double>({N, 3});
                 auto mass = make_array<double>({N});
                 auto tid = make_array<uint32_t>({N});
                 auto img = make_array<int32_t>({N, 3});
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
        .value("DPD", PairKind::DPD);

    py::class_<PairForce, std::shared_ptr<PairForce>>(m, "PotentialPairGPU")
        .def(py::init<std::shared_ptr<ParticleData>, std::shared_ptr<NeighborList>, PairKind>())
        .def("setParamsLJ", &PairForce::set_params_lj)
        .def("setParamsExample", &PairForce::set_params_example)
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
            "mode", [](PairForce& f) { return f.shift_mode; },
            [](PairForce& f, int v) {
                if (v < 0 || v > 2)
                    throw std::invalid_argument("mode must be 0 (none), 1 (shift) or 2 (xplor)");
                f.shift_mode = v;
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

    py::class_<Integrator, std::shared_ptr<Integrator>>(m, "IntegratorTwoStep")
        .def(py::init<std::shared_ptr<ParticleData>, std::shared_ptr<NeighborList>, double>())
        .def("addForce", &Integrator::add_force)
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
                i.prepared = false; // prepare() drops the captured graphs
            })
        .def("prepRun", &Integrator::prepare)
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
