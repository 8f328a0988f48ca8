// Entity's own SR kernels, compiled unmodified from the reference sources
// against the host Kokkos shim in oracle/kokkos_shim (TEST INFRASTRUCTURE).
//
// This translation unit contains no physics of its own: each entry point
// wraps the caller's arrays in shim Views and runs the reference's functor the
// way the reference's host wrapper launches it. The entry points take the
// oracle's grid and species structs (srpic_oracle.h), so the tests can run the
// restated oracle and the reference's code on identical inputs.
//
// Built by oracle/build_ref.py once per (precision, SHAPE_ORDER), because the
// reference fixes both at compile time (cmake/config.cmake:4-28): the shape
// order selects the pusher's interpolation and N_GHOSTS (global.h:130-136).
#include "enums.h"
#include "global.h"

#include "arch/directions.h"
#include "arch/kokkos_aliases.h"
#include "framework/domain/comm_nompi.hpp"
#include "metrics/minkowski.h"
#include "metrics/qkerr_schild.h"
#include "utils/sorting.h"

#include "kernels/ampere_gr.hpp"
#include "kernels/ampere_mink.hpp"
#include "kernels/aux_fields_gr.hpp"
#include "kernels/faraday_gr.hpp"
#include "kernels/fields_bcs.hpp"
#include "kernels/currents_deposit.hpp"
#include "kernels/digital_filter.hpp"
#include "kernels/divergences.hpp"
#include "kernels/faraday_mink.hpp"
#include "kernels/pushers/gr.hpp"
#include "kernels/pushers/sr.hpp"

#include "srpic_oracle.h"

#include <cstdint>
#include <vector>

namespace {
  using namespace ntt;

  template <typename T>
  array_t<T*> wrap1(void* p, std::int64_t n) {
    if (p == nullptr) {
      return array_t<T*> {};
    }
    return array_t<T*>(static_cast<T*>(p), static_cast<std::size_t>(n));
  }

  // ghost-inclusive field of N components with the oracle's strides
  template <Dimension D, unsigned short N>
  ndfield_t<D, N> wrap_field(const orc_grid* g, const void* p, const int64_t* s) {
    const std::size_t ng = (std::size_t)g->ng;
    std::size_t       ext[4], st[4];
    ext[0] = (std::size_t)g->n1 + 2 * ng;
    st[0]  = (std::size_t)s[0];
    ext[1] = (std::size_t)g->n2 + 2 * ng;
    st[1]  = (std::size_t)s[1];
    if constexpr (D == Dim::_3D) {
      ext[2] = (std::size_t)g->n3 + 2 * ng;
      st[2]  = (std::size_t)s[2];
    }
    ext[D] = N;
    st[D]  = (std::size_t)s[3];
    return ndfield_t<D, N>::wrap_strided(static_cast<real_t*>(const_cast<void*>(p)), ext, st);
  }

  template <Dimension D>
  metric::Minkowski<D> make_metric(const orc_grid* g, double dx) {
    std::vector<ncells_t> res { (ncells_t)g->n1, (ncells_t)g->n2 };
    boundaries_t<real_t>  ext { { ZERO, (real_t)g->n1 * (real_t)dx },
                                { ZERO, (real_t)g->n2 * (real_t)dx } };
    if constexpr (D == Dim::_3D) {
      res.push_back((ncells_t)g->n3);
      ext.push_back({ ZERO, (real_t)g->n3 * (real_t)dx });
    }
    return metric::Minkowski<D>(res, ext);
  }

  template <Dimension D>
  range_t<D> active_range(const orc_grid* g) {
    if constexpr (D == Dim::_2D) {
      return range_t<D>({ N_GHOSTS, N_GHOSTS },
                        { N_GHOSTS + (ncells_t)g->n1, N_GHOSTS + (ncells_t)g->n2 });
    } else {
      return range_t<D>({ N_GHOSTS, N_GHOSTS, N_GHOSTS },
                        { N_GHOSTS + (ncells_t)g->n1,
                          N_GHOSTS + (ncells_t)g->n2,
                          N_GHOSTS + (ncells_t)g->n3 });
    }
  }

  PrtlBC prtl_bc(int code) {
    switch (code) {
      case 0:
        return PrtlBC::PERIODIC;
      case 1:
        return PrtlBC::ABSORB;
      case 2:
        return PrtlBC::REFLECT;
      default:
        return PrtlBC::AXIS;
    }
  }

  FldsBC flds_bc(int code) {
    switch (code) {
      case 0:
        return FldsBC::PERIODIC;
      case 2:
        return FldsBC::CONDUCTOR;
      case 3:
        return FldsBC::MATCH;
      default:
        return FldsBC::FIXED;
    }
  }

  ParticleArrays arrays_of(const orc_species* sp) {
    ParticleArrays a;
    const auto     n = sp->npart;
    a.i1             = wrap1<int>(sp->i1, n);
    a.i2             = wrap1<int>(sp->i2, n);
    a.i3             = wrap1<int>(sp->i3, n);
    a.i1_prev        = wrap1<int>(sp->i1_prev, n);
    a.i2_prev        = wrap1<int>(sp->i2_prev, n);
    a.i3_prev        = wrap1<int>(sp->i3_prev, n);
    a.dx1            = wrap1<prtldx_t>(sp->dx1, n);
    a.dx2            = wrap1<prtldx_t>(sp->dx2, n);
    a.dx3            = wrap1<prtldx_t>(sp->dx3, n);
    a.dx1_prev       = wrap1<prtldx_t>(sp->dx1_prev, n);
    a.dx2_prev       = wrap1<prtldx_t>(sp->dx2_prev, n);
    a.dx3_prev       = wrap1<prtldx_t>(sp->dx3_prev, n);
    a.ux1            = wrap1<real_t>(sp->ux1, n);
    a.ux2            = wrap1<real_t>(sp->ux2, n);
    a.ux3            = wrap1<real_t>(sp->ux3, n);
    a.weight         = wrap1<real_t>(sp->weight, n);
    a.tag            = wrap1<short>(sp->tag, n);
    return a;
  }

  // srpic::ParticlePush (src/engines/srpic/particle_pusher.h:35-185) for one
  // species without atmosphere, drag or emission: PusherContext, the particle
  // boundaries of the mesh, the default policy, one parallel_for
  template <Dimension D>
  void push(const orc_grid* g, orc_species* sp, const void* EB, double dt, double omegaB0,
            double dx) {
    using M = metric::Minkowski<D>;
    ParticlePusherFlags flags = ParticlePusher::NONE;
    if (sp->pusher == ORC_PUSHER_BORIS) {
      flags = ParticlePusher::BORIS;
    } else if (sp->pusher == ORC_PUSHER_VAY) {
      flags = ParticlePusher::VAY;
    } else if (sp->pusher == ORC_PUSHER_PHOTON) {
      flags = ParticlePusher::PHOTON;
    }
    if (flags == ParticlePusher::NONE || sp->npart == 0) {
      return;
    }
    kernel::sr::PusherContext ctx { 1u,
                                    flags,
                                    RadiativeDrag::NONE,
                                    sp->mass,
                                    sp->charge,
                                    0.0,
                                    (real_t)dt,
                                    (real_t)omegaB0,
                                    g->n1,
                                    g->n2,
                                    D == Dim::_3D ? g->n3 : 1 };
    boundaries_t<PrtlBC> bcs;
    for (int d = 0; d < (int)D; ++d) {
      bcs.push_back({ prtl_bc(g->prtl_bc[d][0]), prtl_bc(g->prtl_bc[d][1]) });
    }
    kernel::sr::PusherBoundaries<D> bnd { bcs };
    ParticleArrays                  arrays = arrays_of(sp);
    const auto                      em     = wrap_field<D, 6>(g, EB, g->em_s);
    const M                         metric = make_metric<D>(g, dx);
    using P                                = kernel::sr::PusherPolicy<M>;
    Kokkos::parallel_for("ParticlePusher",
                         Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace>(0, sp->npart),
                         kernel::sr::Pusher_kernel<M, P> { ctx, bnd, arrays, em, metric, P {} });
  }

  // srpic::CurrentsDeposit (src/engines/srpic/currents.h:32-87) for one
  // species into J (not zeroed here): a scatter view, the deposit kernel at
  // the build's shape order, contribute
  template <Dimension D>
  void deposit(const orc_grid* g, const orc_species* sp, void* J, double dt, double dx) {
    using M = metric::Minkowski<D>;
    if (sp->npart == 0 || sp->pusher == ORC_PUSHER_NONE || sp->charge == 0.0f) {
      return;
    }
    auto       cur         = wrap_field<D, 3>(g, J, g->cur_s);
    auto       scatter_cur = Kokkos::Experimental::create_scatter_view(cur);
    const auto a           = arrays_of(sp);
    const M    metric      = make_metric<D>(g, dx);
    Kokkos::parallel_for(
      "CurrentsDeposit",
      Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace>(0, sp->npart),
      kernel::DepositCurrents_kernel<SimEngine::SRPIC, M, SHAPE_ORDER>(
        scatter_cur, a.i1, a.i2, a.i3, a.i1_prev, a.i2_prev, a.i3_prev, a.dx1, a.dx2, a.dx3,
        a.dx1_prev, a.dx2_prev, a.dx3_prev, a.ux1, a.ux2, a.ux3, array_t<real_t*> {}, a.weight,
        a.tag, metric, (real_t)sp->charge, (real_t)dt));
    Kokkos::Experimental::contribute(cur, scatter_cur);
  }

  template <Dimension D>
  void faraday(const orc_grid* g, void* EB, double coeff1, double coeff2, const double* st) {
    auto em = wrap_field<D, 6>(g, EB, g->em_s);
    real_t s[9] = { ZERO, ZERO, ZERO, ZERO, ZERO, ZERO, ZERO, ZERO, ZERO };
    if (st != nullptr) {
      for (int k = 0; k < 9; ++k) {
        s[k] = (real_t)st[k];
      }
    }
    Kokkos::parallel_for("Faraday",
                         active_range<D>(g),
                         kernel::mink::Faraday_kernel<D>(em,
                                                         (real_t)coeff1,
                                                         (real_t)coeff2,
                                                         s[0], s[1], s[2], s[3], s[4],
                                                         s[5], s[6], s[7], s[8]));
  }

  template <Dimension D>
  void ampere(const orc_grid* g, void* EB, double coeff1, double coeff2) {
    auto em = wrap_field<D, 6>(g, EB, g->em_s);
    Kokkos::parallel_for("Ampere",
                         active_range<D>(g),
                         kernel::mink::Ampere_kernel<D>(em, (real_t)coeff1, (real_t)coeff2));
  }

  template <Dimension D>
  void currents_ampere(const orc_grid* g, void* EB, void* J, double coeff, double ppc0) {
    auto em  = wrap_field<D, 6>(g, EB, g->em_s);
    auto cur = wrap_field<D, 3>(g, J, g->cur_s);
    Kokkos::parallel_for("Ampere",
                         active_range<D>(g),
                         kernel::mink::CurrentsAmpere_kernel<D>(em, cur, (real_t)coeff,
                                                                (real_t)ppc0));
  }

  // one pass of srpic::CurrentsFilter (src/engines/srpic/currents.h:89-119)
  // without the ghost exchange that follows it
  template <Dimension D>
  void filter_pass(const orc_grid* g, void* J, void* buff) {
    auto cur = wrap_field<D, 3>(g, J, g->cur_s);
    auto buf = wrap_field<D, 3>(g, buff, g->cur_s);
    ncells_t size[D];
    size[0] = (ncells_t)g->n1;
    size[1] = (ncells_t)g->n2;
    if constexpr (D == Dim::_3D) {
      size[2] = (ncells_t)g->n3;
    }
    boundaries_t<FldsBC> bcs;
    for (int d = 0; d < (int)D; ++d) {
      bcs.push_back({ flds_bc(g->fbc[d][0]), flds_bc(g->fbc[d][1]) });
    }
    Kokkos::deep_copy(buf, cur);
    Kokkos::parallel_for("CurrentsFilter",
                         active_range<D>(g),
                         kernel::DigitalFilter_kernel<D, Coord::Cartesian>(cur, buf, size, bcs));
  }

  // one pass of grpic::CurrentsFilter (src/engines/grpic/currents.h:74-101)
  // on a 2D non-Cartesian grid: the range runs one row past the last active
  // row (the upper axis row); the radial sides are not filtered specially
  void filter_pass_axisym(const orc_grid* g, void* J, void* buff, int axis_min, int axis_max) {
    auto cur = wrap_field<Dim::_2D, 3>(g, J, g->cur_s);
    auto buf = wrap_field<Dim::_2D, 3>(g, buff, g->cur_s);
    ncells_t size[2] = { (ncells_t)g->n1, (ncells_t)g->n2 };
    boundaries_t<FldsBC> bcs = { { FldsBC::HORIZON, FldsBC::MATCH },
                                 { axis_min ? FldsBC::AXIS : FldsBC::FIXED,
                                   axis_max ? FldsBC::AXIS : FldsBC::FIXED } };
    Kokkos::deep_copy(buf, cur);
    Kokkos::parallel_for(
      "CurrentsFilter",
      range_t<Dim::_2D>({ N_GHOSTS, N_GHOSTS },
                        { N_GHOSTS + (ncells_t)g->n1, N_GHOSTS + (ncells_t)g->n2 + 1 }),
      kernel::DigitalFilter_kernel<Dim::_2D, Coord::Qspherical>(cur, buf, size, bcs));
  }

  // sort::PositionToTileIndex<D, false> with tile size 1 (the key of
  // Particles::SortSpatially, src/framework/containers/particles_sort.cpp:196-253)
  template <Dimension D>
  void sort_keys(const orc_grid* g, const orc_species* sp, std::uint32_t* keys) {
    const auto          a = arrays_of(sp);
    array_t<ncells_t*>  k(reinterpret_cast<ncells_t*>(keys), (std::size_t)sp->npart);
    std::vector<ncells_t> n { (ncells_t)g->n1, (ncells_t)g->n2 };
    if constexpr (D == Dim::_3D) {
      n.push_back((ncells_t)g->n3);
    }
    sort::PositionToTileIndex<D, false> f(a.i1, a.i2, a.i3, a.tag, k, n, 1u);
    Kokkos::parallel_for("Keys",
                         Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace>(0, sp->npart),
                         f);
  }

  // ---- field exchange of one periodic domain -----------------------------
  // Metadomain::CommunicateFields / SynchronizeFields (metadomain_comm.cpp:
  // 204-367, 408-562) for a domain that is its own neighbour along every
  // periodic axis: the send and receive slices of GetSendRecvParams
  // (metadomain_comm.cpp:117-193) around the reference's
  // comm::CommunicateField (comm_nompi.hpp), over dir::Directions<D>::all. A
  // direction with a component along a non-periodic axis has no neighbour
  // and is skipped, as GetSendRecvRanks leaves it.
  template <Dimension D>
  bool exchange_slices(const orc_grid* g, const dir::direction_t<D>& dir, bool synchronize,
                       std::vector<cell_range_t>& send, std::vector<cell_range_t>& recv) {
    const int n[3] = { g->n1, g->n2, g->n3 };
    for (auto d { 0u }; d < dir.size(); ++d) {
      if (dir[d] != 0 && !g->periodic[d]) {
        return false;
      }
    }
    for (auto d { 0u }; d < dir.size(); ++d) {
      const ncells_t imin = N_GHOSTS, imax = N_GHOSTS + (ncells_t)n[d];
      const int      dr = dir[d];
      if (!synchronize) {
        // send from the active zones, receive into the ghost zones
        send.emplace_back(dr == 0 ? imin : (dr == 1 ? imax - N_GHOSTS : imin),
                          dr == 0 ? imax : (dr == 1 ? imax : imin + N_GHOSTS));
        recv.emplace_back(-dr == 0 ? imin : (-dr == 1 ? imax : imin - N_GHOSTS),
                          -dr == 0 ? imax : (-dr == 1 ? imax + N_GHOSTS : imin));
      } else {
        // send from and receive into active + ghost zones
        send.emplace_back(dr == 0 ? imin - N_GHOSTS : (dr == 1 ? imax - N_GHOSTS : imin - N_GHOSTS),
                          dr == 0 ? imax + N_GHOSTS : (dr == 1 ? imax + N_GHOSTS : imin + N_GHOSTS));
        recv.emplace_back(-dr == 0 ? imin - N_GHOSTS : (-dr == 1 ? imax - N_GHOSTS : imin - N_GHOSTS),
                          -dr == 0 ? imax + N_GHOSTS : (-dr == 1 ? imax + N_GHOSTS : imin + N_GHOSTS));
      }
    }
    return true;
  }

  template <Dimension D, unsigned short N>
  void communicate(const orc_grid* g, void* fld, const int64_t* s, int c0, int c1) {
    auto f = wrap_field<D, N>(g, fld, s);
    for (const auto& dir : dir::Directions<D>::all) {
      std::vector<cell_range_t> send, recv;
      if (!exchange_slices<D>(g, dir, false, send, recv)) {
        continue;
      }
      comm::CommunicateField<D, N>(0, f, f, 0, 0, 0, 0, send, recv,
                                   cell_range_t((ncells_t)c0, (ncells_t)c1), false);
    }
  }

  template <Dimension D>
  void synchronize_currents(const orc_grid* g, void* J, void* buff) {
    auto cur = wrap_field<D, 3>(g, J, g->cur_s);
    auto bf  = wrap_field<D, 3>(g, buff, g->cur_s);
    Kokkos::deep_copy(bf, ZERO);
    for (const auto& dir : dir::Directions<D>::all) {
      std::vector<cell_range_t> send, recv;
      if (!exchange_slices<D>(g, dir, true, send, recv)) {
        continue;
      }
      comm::CommunicateField<D, 3>(0, cur, bf, 0, 0, 0, 0, send, recv, cell_range_t(0, 3), true);
    }
    // AddBufferedFields over the active cells (metadomain_comm.cpp:370-406)
    const std::size_t ng = N_GHOSTS;
    if constexpr (D == Dim::_2D) {
      for (std::size_t i = ng; i < ng + (std::size_t)g->n1; ++i)
        for (std::size_t j = ng; j < ng + (std::size_t)g->n2; ++j)
          for (int c = 0; c < 3; ++c) cur(i, j, c) += bf(i, j, c);
    } else {
      for (std::size_t i = ng; i < ng + (std::size_t)g->n1; ++i)
        for (std::size_t j = ng; j < ng + (std::size_t)g->n2; ++j)
          for (std::size_t k = ng; k < ng + (std::size_t)g->n3; ++k)
            for (int c = 0; c < 3; ++c) cur(i, j, k, c) += bf(i, j, k, c);
    }
  }

  // ---- SR perfect-conductor walls ----------------------------------------
  // srpic::FieldBoundaries (srpic/fields_bcs.h:622-672) for the CONDUCTOR
  // sides, in Directions<D>::orth order: PerfectConductorFieldsIn's range
  // (fields_bcs.h:356-396: the ghost layers and the edge, N_GHOSTS + 1 cells
  // on the lower side) and ConductorBoundaries_kernel (fields_bcs.hpp:523-800)
  template <Dimension D, in O, bool P>
  void conductor_side(const orc_grid* g, ndfield_t<D, 6>& em, ncells_t i_edge, BCTags tags,
                      const std::int64_t* lo, const std::int64_t* hi) {
    if constexpr (D == Dim::_2D) {
      Kokkos::parallel_for(Kokkos::MDRangePolicy<Kokkos::Rank<2>>({ lo[0], lo[1] }, { hi[0], hi[1] }),
                           kernel::bc::ConductorBoundaries_kernel<D, O, P>(em, i_edge, tags));
    } else {
      Kokkos::parallel_for(
        Kokkos::MDRangePolicy<Kokkos::Rank<3>>({ lo[0], lo[1], lo[2] }, { hi[0], hi[1], hi[2] }),
        kernel::bc::ConductorBoundaries_kernel<D, O, P>(em, i_edge, tags));
    }
  }

  template <Dimension D>
  void conductor_walls(const orc_grid* g, void* EB, int set_e, int set_b) {
    auto         em   = wrap_field<D, 6>(g, EB, g->em_s);
    const BCTags tags = (set_e ? (BCTags)BC::E : (BCTags)0) | (set_b ? (BCTags)BC::B : (BCTags)0);
    const int    n[3] = { g->n1, g->n2, g->n3 };
    for (const auto& dir : dir::Directions<D>::orth) {
      const auto sign = dir.get_sign();
      const int  d    = (int)dir.get_dim();
      if (g->fbc[d][sign > 0 ? 1 : 0] != 2) {
        continue;
      }
      std::int64_t lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
      for (int a = 0; a < (int)D; ++a) {
        hi[a] = (a == d) ? (sign < 0 ? N_GHOSTS + 1 : N_GHOSTS) : n[a] + 2 * N_GHOSTS;
      }
      const ncells_t i_edge = sign > 0 ? N_GHOSTS + (ncells_t)n[d] : N_GHOSTS;
      if (d == 0) {
        if (sign > 0) conductor_side<D, in::x1, true>(g, em, i_edge, tags, lo, hi);
        else          conductor_side<D, in::x1, false>(g, em, i_edge, tags, lo, hi);
      } else if (d == 1) {
        if (sign > 0) conductor_side<D, in::x2, true>(g, em, i_edge, tags, lo, hi);
        else          conductor_side<D, in::x2, false>(g, em, i_edge, tags, lo, hi);
      } else if constexpr (D == Dim::_3D) {
        if (sign > 0) conductor_side<D, in::x3, true>(g, em, i_edge, tags, lo, hi);
        else          conductor_side<D, in::x3, false>(g, em, i_edge, tags, lo, hi);
      }
    }
  }

  // ---- output: div E -------------------------------------------------------
  // ComputeDivergence_kernel<Minkowski, 6> over the active cells into
  // component `comp` of a 6-component buffer (metadomain_io.cpp:525-533)
  template <Dimension D>
  void divergence(const orc_grid* g, const void* EB, void* bckp, int comp, double dx) {
    auto       em  = wrap_field<D, 6>(g, EB, g->em_s);
    auto       out = wrap_field<D, 6>(g, bckp, g->em_s);
    const auto metric = make_metric<D>(g, dx);
    const std::int64_t ng = N_GHOSTS;
    if constexpr (D == Dim::_2D) {
      Kokkos::parallel_for(
        Kokkos::MDRangePolicy<Kokkos::Rank<2>>({ ng, ng }, { ng + g->n1, ng + g->n2 }),
        kernel::ComputeDivergence_kernel<metric::Minkowski<D>, 6>(metric, em, out, (idx_t)comp));
    } else {
      Kokkos::parallel_for(
        Kokkos::MDRangePolicy<Kokkos::Rank<3>>({ ng, ng, ng }, { ng + g->n1, ng + g->n2, ng + g->n3 }),
        kernel::ComputeDivergence_kernel<metric::Minkowski<D>, 6>(metric, em, out, (idx_t)comp));
    }
  }

  // ---- GR: metric::QKerrSchild<Dim::_2D> --------------------------------
  // mp = { x1min, x1max, x2min, x2max, a, r0, h }
  using QKS = metric::QKerrSchild<Dim::_2D>;
  QKS make_qks(int n1, int n2, const double* mp) {
    std::vector<ncells_t> res { (ncells_t)n1, (ncells_t)n2 };
    boundaries_t<real_t>  ext { { (real_t)mp[0], (real_t)mp[1] }, { (real_t)mp[2], (real_t)mp[3] } };
    std::map<std::string, real_t> prm { { "a", (real_t)mp[4] }, { "r0", (real_t)mp[5] },
                                        { "h", (real_t)mp[6] } };
    return QKS(res, ext, prm);
  }

  // grpic::ParticlePush (src/engines/grpic/particle_pusher.h:26-94) for one
  // species
  void gr_push(const orc_grid* g, const double* mp, orc_species* sp, const void* em,
               const void* em0, double dt, double omegaB0, int niter, const int* absorb,
               const int* axis) {
    if (sp->npart == 0 || sp->pusher == ORC_PUSHER_NONE) {
      return;
    }
    const QKS                  metric = make_qks(g->n1, g->n2, mp);
    const kernel::gr::PusherContext ctx { sp->mass,
                                          sp->charge,
                                          (real_t)dt,
                                          (real_t)omegaB0,
                                          (real_t)1e-6,
                                          (unsigned short)niter,
                                          g->n1,
                                          g->n2,
                                          1 };
    boundaries_t<PrtlBC> bcs { { absorb[0] ? PrtlBC::ABSORB : PrtlBC::PERIODIC,
                                 absorb[1] ? PrtlBC::ABSORB : PrtlBC::PERIODIC },
                               { axis[0] ? PrtlBC::AXIS : PrtlBC::PERIODIC,
                                 axis[1] ? PrtlBC::AXIS : PrtlBC::PERIODIC } };
    const kernel::gr::PusherBoundaries<Dim::_2D> bnd { bcs };
    ParticleArrays arrays = arrays_of(sp);
    const auto     DB     = wrap_field<Dim::_2D, 6>(g, em, g->em_s);
    const auto     DB0    = wrap_field<Dim::_2D, 6>(g, em0, g->em_s);
    kernel::gr::Pusher_kernel<QKS> k(ctx, bnd, arrays, DB, DB0, metric);
    if (sp->pusher == ORC_PUSHER_PHOTON) {
      Kokkos::parallel_for(
        "ParticlePusher",
        Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace, kernel::gr::Massless_t>(0, sp->npart),
        k);
    } else {
      Kokkos::parallel_for(
        "ParticlePusher",
        Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace, kernel::gr::Massive_t>(0, sp->npart),
        k);
    }
  }

  // grpic::CurrentsDeposit (src/engines/grpic/currents.h:29-73): order 1
  void gr_deposit(const orc_grid* g, const double* mp, const orc_species* sp, void* J,
                  double dt) {
    if (sp->npart == 0 || sp->pusher == ORC_PUSHER_NONE || sp->charge == 0.0f) {
      return;
    }
    const QKS  metric      = make_qks(g->n1, g->n2, mp);
    auto       cur         = wrap_field<Dim::_2D, 3>(g, J, g->cur_s);
    auto       scatter_cur = Kokkos::Experimental::create_scatter_view(cur);
    const auto a           = arrays_of(sp);
    Kokkos::parallel_for(
      "CurrentsDeposit",
      Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace>(0, sp->npart),
      kernel::DepositCurrents_kernel<SimEngine::GRPIC, QKS>(
        scatter_cur, a.i1, a.i2, a.i3, a.i1_prev, a.i2_prev, a.i3_prev, a.dx1, a.dx2, a.dx3,
        a.dx1_prev, a.dx2_prev, a.dx3_prev, a.ux1, a.ux2, a.ux3, array_t<real_t*> {}, a.weight,
        a.tag, metric, (real_t)sp->charge, (real_t)dt));
    Kokkos::Experimental::contribute(cur, scatter_cur);
  }

  boundaries_t<FldsBC> gr_flds_bc(int axis_min, int axis_max, int horizon) {
    return { { horizon ? FldsBC::HORIZON : FldsBC::FIXED, FldsBC::MATCH },
             { axis_min ? FldsBC::AXIS : FldsBC::FIXED, axis_max ? FldsBC::AXIS : FldsBC::FIXED } };
  }

  range_t<Dim::_2D> gr_range(const orc_grid* g, int di1_lo, int di2_hi) {
    return range_t<Dim::_2D>({ N_GHOSTS - di1_lo, N_GHOSTS },
                             { N_GHOSTS + (ncells_t)g->n1, N_GHOSTS + (ncells_t)g->n2 + di2_hi });
  }

  // the GR field kernels as grpic/fieldsolvers.h:79-266 and grpic/utils.h
  // launch them: op 0 Faraday (a = Bin, b = Bout, c = E), 1 Ampere (a = Din,
  // b = Dout, c = H), 2 CurrentsAmpere (a = D, c = J), 3 ComputeAuxE (a = D,
  // b = B, c = E), 4 ComputeAuxH (a = D, b = B, c = H), 5 TimeAverageDB
  // (a = em, b = em0), 6 TimeAverageJ (a = cur, b = cur0)
  void gr_field(const orc_grid* g, const double* mp, int op, void* a, void* b, void* c,
                double coeff, int axis_min, int axis_max) {
    const QKS  metric = make_qks(g->n1, g->n2, mp);
    const auto bcs    = gr_flds_bc(axis_min, axis_max, 1);
    const auto ni2    = (ncells_t)g->n2;
    auto       em     = [&](void* p) { return wrap_field<Dim::_2D, 6>(g, p, g->em_s); };
    auto       cu     = [&](void* p) { return wrap_field<Dim::_2D, 3>(g, p, g->cur_s); };
    switch (op) {
      case 0:
        Kokkos::parallel_for("Faraday", gr_range(g, 0, 0),
                             kernel::gr::Faraday_kernel<QKS>(em(a), em(b), em(c), metric,
                                                             (real_t)coeff, ni2, bcs));
        break;
      case 1:
        Kokkos::parallel_for("Ampere", gr_range(g, 0, 1),
                             kernel::gr::Ampere_kernel<QKS>(em(a), em(b), em(c), metric,
                                                            (real_t)coeff, ni2, bcs));
        break;
      case 2:
        Kokkos::parallel_for("AmpereCurrents", gr_range(g, 0, 1),
                             kernel::gr::CurrentsAmpere_kernel<QKS>(em(a), cu(c), metric,
                                                                    (real_t)coeff, ni2, bcs));
        break;
      case 3:
        Kokkos::parallel_for("ComputeAuxE", gr_range(g, 1, axis_max ? 1 : 0),
                             kernel::gr::ComputeAuxE_kernel<QKS>(em(a), em(b), em(c), metric));
        break;
      case 4:
        Kokkos::parallel_for("ComputeAuxH", gr_range(g, 1, axis_max ? 1 : 0),
                             kernel::gr::ComputeAuxH_kernel<QKS>(em(a), em(b), em(c), metric));
        break;
      case 5:
        Kokkos::parallel_for("TimeAverageDB", gr_range(g, 0, 0),
                             kernel::gr::TimeAverageDB_kernel<Dim::_2D>(em(a), em(b)));
        break;
      case 6:
        Kokkos::parallel_for("TimeAverageJ", gr_range(g, 0, 0),
                             kernel::gr::TimeAverageJ_kernel<Dim::_2D>(cu(a), cu(b)));
        break;
      default:
        break;
    }
  }

  // grpic::FieldBoundaries(gr_bc::main) on one field for the horizon and the
  // axes, in Directions<2>::orth order: -x1 (horizon), -x2, +x2 (axes)
  // (src/engines/grpic/fields_bcs.h:138-222, 238-252)
  void gr_field_bcs(const orc_grid* g, void* fld, int set_e, int set_b, int axis_min,
                    int axis_max, int horizon, int nfilter) {
    auto         F    = wrap_field<Dim::_2D, 6>(g, fld, g->em_s);
    const BCTags tags = (set_e ? (BC::Ex1 | BC::Ex2 | BC::Ex3) : 0) |
                        (set_b ? (BC::Bx1 | BC::Bx2 | BC::Bx3) : 0);
    const ncells_t i1min = N_GHOSTS, i2min = N_GHOSTS, i2max = N_GHOSTS + (ncells_t)g->n2;
    if (horizon) {
      Kokkos::parallel_for("OpenBCFields", range_t<Dim::_1D>(i2min, i2max + 1),
                           kernel::bc::gr::HorizonBoundaries_kernel<Dim::_2D>(F, i1min, tags,
                                                                                (unsigned short)nfilter));
    }
    const auto n_all1 = (ncells_t)(g->n1 + 2 * g->ng);
    if (axis_min) {
      Kokkos::parallel_for("AxisBCFields", n_all1,
                           kernel::bc::AxisBoundaries_kernel<Dim::_2D, false>(F, i2min, tags));
    }
    if (axis_max) {
      Kokkos::parallel_for("AxisBCFields", n_all1,
                           kernel::bc::AxisBoundaries_kernel<Dim::_2D, true>(F, i2max, tags));
    }
  }

  template <class F2, class F3>
  int dispatch(const orc_grid* g, F2&& f2, F3&& f3) {
    if (g->ng != (int)N_GHOSTS) {
      return -2;
    }
    if (g->dim == 2) {
      f2();
    } else if (g->dim == 3) {
      f3();
    } else {
      return -1;
    }
    return 0;
  }
} // namespace

static_assert(sizeof(ncells_t) == 4, "sort keys are 32-bit");

extern "C" {

int ref_shape_order(void) {
  return SHAPE_ORDER;
}

int ref_n_ghosts(void) {
  return (int)N_GHOSTS;
}

int ref_real_size(void) {
  return (int)sizeof(real_t);
}

int ref_push(const orc_grid* g, orc_species* sp, const void* EB, double dt, double omegaB0,
             double dx) {
  return dispatch(
    g,
    [&] { push<Dim::_2D>(g, sp, EB, dt, omegaB0, dx); },
    [&] { push<Dim::_3D>(g, sp, EB, dt, omegaB0, dx); });
}

int ref_deposit(const orc_grid* g, const orc_species* sp, void* J, double dt, double dx) {
  return dispatch(
    g,
    [&] { deposit<Dim::_2D>(g, sp, J, dt, dx); },
    [&] { deposit<Dim::_3D>(g, sp, J, dt, dx); });
}

int ref_faraday(const orc_grid* g, void* EB, double coeff1, double coeff2,
                const double* stencil) {
  return dispatch(
    g,
    [&] { faraday<Dim::_2D>(g, EB, coeff1, coeff2, stencil); },
    [&] { faraday<Dim::_3D>(g, EB, coeff1, coeff2, stencil); });
}

int ref_ampere(const orc_grid* g, void* EB, double coeff1, double coeff2) {
  return dispatch(
    g,
    [&] { ampere<Dim::_2D>(g, EB, coeff1, coeff2); },
    [&] { ampere<Dim::_3D>(g, EB, coeff1, coeff2); });
}

int ref_currents_ampere(const orc_grid* g, void* EB, void* J, double coeff, double ppc0) {
  return dispatch(
    g,
    [&] { currents_ampere<Dim::_2D>(g, EB, J, coeff, ppc0); },
    [&] { currents_ampere<Dim::_3D>(g, EB, J, coeff, ppc0); });
}

// CommunicateFields on a field of the em (is_em) or cur layout, components
// [c0, c1): the ghost zones refilled from the active zones
int ref_communicate(const orc_grid* g, void* fld, int is_em, int c0, int c1) {
  return dispatch(
    g,
    [&] {
      if (is_em) communicate<Dim::_2D, 6>(g, fld, g->em_s, c0, c1);
      else       communicate<Dim::_2D, 3>(g, fld, g->cur_s, c0, c1);
    },
    [&] {
      if (is_em) communicate<Dim::_3D, 6>(g, fld, g->em_s, c0, c1);
      else       communicate<Dim::_3D, 3>(g, fld, g->cur_s, c0, c1);
    });
}

// div E of EB into component comp of bckp (em layout), active cells
int ref_output_divergence(const orc_grid* g, const void* EB, void* bckp, int comp, double dx) {
  return dispatch(
    g, [&] { divergence<Dim::_2D>(g, EB, bckp, comp, dx); },
    [&] { divergence<Dim::_3D>(g, EB, bckp, comp, dx); });
}

// the perfect-conductor sides of g->fbc (2) on EB
int ref_conductor_walls(const orc_grid* g, void* EB, int set_e, int set_b) {
  return dispatch(
    g, [&] { conductor_walls<Dim::_2D>(g, EB, set_e, set_b); },
    [&] { conductor_walls<Dim::_3D>(g, EB, set_e, set_b); });
}

// SynchronizeFields(J): the additive fold of J's ghost and edge zones
int ref_sync_currents(const orc_grid* g, void* J, void* buff) {
  return dispatch(
    g, [&] { synchronize_currents<Dim::_2D>(g, J, buff); },
    [&] { synchronize_currents<Dim::_3D>(g, J, buff); });
}

int ref_filter_pass(const orc_grid* g, void* J, void* buff) {
  return dispatch(
    g,
    [&] { filter_pass<Dim::_2D>(g, J, buff); },
    [&] { filter_pass<Dim::_3D>(g, J, buff); });
}

int ref_filter_pass_axisym(const orc_grid* g, void* J, void* buff, int axis_min, int axis_max) {
  if (g->ng != (int)N_GHOSTS || g->dim != 2) {
    return -1;
  }
  filter_pass_axisym(g, J, buff, axis_min, axis_max);
  return 0;
}

// the QKerrSchild metric functions at n points x (n x 2 code coordinates),
// out (n x 24) in the oracle's order (grpic_oracle.h: h_11 h_22 h_33 h_13 h11
// h22 h33 h13 alpha beta1 sqrt_det_h sqrt_det_h_tilde dr_alpha dt_alpha
// dr_beta1 dt_beta1 dr_h11 dr_h22 dr_h33 dr_h13 dt_h11 dt_h22 dt_h33 dt_h13)
int ref_gr_metric(int n1, int n2, const double* mp, const double* x, int64_t n, double* out) {
  const QKS m = make_qks(n1, n2, mp);
  for (int64_t p = 0; p < n; ++p) {
    const coord_t<Dim::_2D> xc { (real_t)x[2 * p], (real_t)x[2 * p + 1] };
    double*                 o = out + 24 * p;
    o[0]  = m.template h_<1, 1>(xc);
    o[1]  = m.template h_<2, 2>(xc);
    o[2]  = m.template h_<3, 3>(xc);
    o[3]  = m.template h_<1, 3>(xc);
    o[4]  = m.template h<1, 1>(xc);
    o[5]  = m.template h<2, 2>(xc);
    o[6]  = m.template h<3, 3>(xc);
    o[7]  = m.template h<1, 3>(xc);
    o[8]  = m.alpha(xc);
    o[9]  = m.beta1(xc);
    o[10] = m.sqrt_det_h(xc);
    o[11] = m.sqrt_det_h_tilde(xc);
    o[12] = m.dr_alpha(xc);
    o[13] = m.dt_alpha(xc);
    o[14] = m.dr_beta1(xc);
    o[15] = m.dt_beta1(xc);
    o[16] = m.dr_h11(xc);
    o[17] = m.dr_h22(xc);
    o[18] = m.dr_h33(xc);
    o[19] = m.dr_h13(xc);
    o[20] = m.dt_h11(xc);
    o[21] = m.dt_h22(xc);
    o[22] = m.dt_h33(xc);
    o[23] = m.dt_h13(xc);
  }
  return 0;
}

// metric.convert<2, Ph, Cd> (to_code = 1: theta -> code x2) or
// convert<2, Cd, Ph> (to_code = 0) at n points (qkerr_schild.h:615-649)
int ref_gr_convert_x2(int n1, int n2, const double* mp, int to_code, const double* in, int64_t n,
                      double* out) {
  const QKS m = make_qks(n1, n2, mp);
  for (int64_t p = 0; p < n; ++p) {
    out[p] = to_code ? m.template convert<2, Crd::Ph, Crd::Cd>((real_t)in[p])
                     : m.template convert<2, Crd::Cd, Crd::Ph>((real_t)in[p]);
  }
  return 0;
}

int ref_gr_push(const orc_grid* g, const double* mp, orc_species* sp, const void* em,
                const void* em0, double dt, double omegaB0, int niter, const int* absorb,
                const int* axis) {
  if (g->ng != (int)N_GHOSTS || g->dim != 2) {
    return -1;
  }
  gr_push(g, mp, sp, em, em0, dt, omegaB0, niter, absorb, axis);
  return 0;
}

int ref_gr_deposit(const orc_grid* g, const double* mp, const orc_species* sp, void* J,
                   double dt) {
  if (g->ng != (int)N_GHOSTS || g->dim != 2) {
    return -1;
  }
  gr_deposit(g, mp, sp, J, dt);
  return 0;
}

int ref_gr_field(const orc_grid* g, const double* mp, int op, void* a, void* b, void* c,
                 double coeff, int axis_min, int axis_max) {
  if (g->ng != (int)N_GHOSTS || g->dim != 2) {
    return -1;
  }
  gr_field(g, mp, op, a, b, c, coeff, axis_min, axis_max);
  return 0;
}

int ref_gr_field_bcs(const orc_grid* g, void* fld, int set_e, int set_b, int axis_min,
                     int axis_max, int horizon, int nfilter) {
  if (g->ng != (int)N_GHOSTS || g->dim != 2) {
    return -1;
  }
  gr_field_bcs(g, fld, set_e, set_b, axis_min, axis_max, horizon, nfilter);
  return 0;
}

int ref_sort_keys(const orc_grid* g, const orc_species* sp, std::uint32_t* keys) {
  return dispatch(
    g,
    [&] { sort_keys<Dim::_2D>(g, sp, keys); },
    [&] { sort_keys<Dim::_3D>(g, sp, keys); });
}

} // extern "C"
