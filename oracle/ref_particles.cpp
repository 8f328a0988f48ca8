// The reference's own particle container on the host Kokkos shim (TEST
// INFRASTRUCTURE ONLY), with a species copied into an
// ntt::Particles<D, Cartesian> (particles.cpp):
//  - Particles::RemoveDead and Particles::SortSpatially
//    (src/framework/containers/particles_sort.cpp:103-253), the species
//    copied back in the new order;
//  - the output moments: ParticleMoments_kernel<SRPIC, Minkowski<D>, F, 6>
//    (src/kernels/particle_moments.hpp:44-405) launched over the species as
//    ComputeMoments launches it (src/framework/domain/metadomain_io.cpp:
//    122-171), scattered into a 6-component buffer.
// Built with the reference's container and grid sources by
// oracle/build_ref.py; adds no logic of its own.
//
// The shim runs these calls serially in index order (Kokkos::shim::g_serial):
// RemoveDead hands out the alive slots with an atomic counter, BinSort fills
// each bin in element order, and the moments' scatter view adds the particles
// in index order, which is what a serial host gives. Kokkos leaves these
// orders to the backend.
#include "enums.h"
#include "global.h"

#include "arch/kokkos_aliases.h"

#include "framework/containers/particles.h"
#include "framework/domain/grid.h"
#include "kernels/particle_moments.hpp"
#include "metrics/minkowski.h"

#include "srpic_oracle.h"

#include <cstdint>
#include <vector>

namespace {
  using namespace ntt;

  template <Dimension D>
  std::int64_t sort_species(const orc_grid* g, orc_species* sp, int remove_dead, real_t* pld_r,
                            int npld_r, std::uint32_t* pld_i, int npld_i) {
    const npart_t n = static_cast<npart_t>(sp->npart);
    ntt::Particles<D, ntt::Coord::Cartesian> p(1, "ref", sp->mass, sp->charge, n > 0 ? n : 1, 0, 0,
                                               ntt::ParticlePusher::BORIS, false,
                                               ntt::RadiativeDrag::NONE, ntt::EmissionType::NONE,
                                               static_cast<unsigned short>(npld_r),
                                               static_cast<unsigned short>(npld_i));
    auto* ux1 = static_cast<real_t*>(sp->ux1);
    auto* ux2 = static_cast<real_t*>(sp->ux2);
    auto* ux3 = static_cast<real_t*>(sp->ux3);
    auto* w   = static_cast<real_t*>(sp->weight);
    for (npart_t k = 0; k < n; ++k) {
      p.i1(k) = sp->i1[k], p.dx1(k) = sp->dx1[k];
      p.i1_prev(k) = sp->i1_prev[k], p.dx1_prev(k) = sp->dx1_prev[k];
      p.i2(k) = sp->i2[k], p.dx2(k) = sp->dx2[k];
      p.i2_prev(k) = sp->i2_prev[k], p.dx2_prev(k) = sp->dx2_prev[k];
      if constexpr (D == Dim::_3D) {
        p.i3(k) = sp->i3[k], p.dx3(k) = sp->dx3[k];
        p.i3_prev(k) = sp->i3_prev[k], p.dx3_prev(k) = sp->dx3_prev[k];
      }
      p.ux1(k) = ux1[k], p.ux2(k) = ux2[k], p.ux3(k) = ux3[k];
      p.weight(k) = w[k];
      p.tag(k)    = sp->tag[k];
      for (int c = 0; c < npld_r; ++c) p.pld_r(k, c) = pld_r[(std::size_t)k * npld_r + c];
      for (int c = 0; c < npld_i; ++c) p.pld_i(k, c) = pld_i[(std::size_t)k * npld_i + c];
    }
    p.set_npart(n);
    std::vector<ncells_t> res { static_cast<ncells_t>(g->n1), static_cast<ncells_t>(g->n2) };
    boundaries_t<real_t>  ext { { ZERO, static_cast<real_t>(g->n1) },
                                { ZERO, static_cast<real_t>(g->n2) } };
    if constexpr (D == Dim::_3D) {
      res.push_back(static_cast<ncells_t>(g->n3));
      ext.push_back({ ZERO, static_cast<real_t>(g->n3) });
    }
    const ntt::Grid<D> grid(res, ext);
    Kokkos::shim::g_serial = true;
    if (remove_dead) {
      p.RemoveDead();
    }
    p.SortSpatially(grid);
    Kokkos::shim::g_serial = false;
    const npart_t m = p.npart();
    for (npart_t k = 0; k < m; ++k) {
      sp->i1[k] = p.i1(k), sp->dx1[k] = p.dx1(k);
      sp->i1_prev[k] = p.i1_prev(k), sp->dx1_prev[k] = p.dx1_prev(k);
      sp->i2[k] = p.i2(k), sp->dx2[k] = p.dx2(k);
      sp->i2_prev[k] = p.i2_prev(k), sp->dx2_prev[k] = p.dx2_prev(k);
      if constexpr (D == Dim::_3D) {
        sp->i3[k] = p.i3(k), sp->dx3[k] = p.dx3(k);
        sp->i3_prev[k] = p.i3_prev(k), sp->dx3_prev[k] = p.dx3_prev(k);
      }
      ux1[k] = p.ux1(k), ux2[k] = p.ux2(k), ux3[k] = p.ux3(k);
      w[k]        = p.weight(k);
      sp->tag[k]  = p.tag(k);
      for (int c = 0; c < npld_r; ++c) pld_r[(std::size_t)k * npld_r + c] = p.pld_r(k, c);
      for (int c = 0; c < npld_i; ++c) pld_i[(std::size_t)k * npld_i + c] = p.pld_i(k, c);
    }
    return static_cast<std::int64_t>(m);
  }

  // the species' arrays copied into a container built for it
  template <Dimension D>
  void fill(ntt::Particles<D, ntt::Coord::Cartesian>& p, const orc_species* sp) {
    const npart_t n   = static_cast<npart_t>(sp->npart);
    const auto* ux1 = static_cast<const real_t*>(sp->ux1);
    const auto* ux2 = static_cast<const real_t*>(sp->ux2);
    const auto* ux3 = static_cast<const real_t*>(sp->ux3);
    const auto* w   = static_cast<const real_t*>(sp->weight);
    for (npart_t k = 0; k < n; ++k) {
      p.i1(k) = sp->i1[k], p.dx1(k) = sp->dx1[k];
      p.i2(k) = sp->i2[k], p.dx2(k) = sp->dx2[k];
      if constexpr (D == Dim::_3D) {
        p.i3(k) = sp->i3[k], p.dx3(k) = sp->dx3[k];
      }
      p.ux1(k) = ux1[k], p.ux2(k) = ux2[k], p.ux3(k) = ux3[k];
      p.weight(k) = w[k];
      p.tag(k)    = sp->tag[k];
    }
    p.set_npart(n);
  }

  // a 6-component ghost-inclusive field with the oracle's em strides
  template <Dimension D>
  ndfield_t<D, 6> wrap_em(const orc_grid* g, void* p) {
    const std::size_t ng = (std::size_t)g->ng;
    std::size_t       ext[4], st[4];
    const int         n[3] = { g->n1, g->n2, g->n3 };
    for (int d = 0; d < (int)D; ++d) {
      ext[d] = (std::size_t)n[d] + 2 * ng;
      st[d]  = (std::size_t)g->em_s[d];
    }
    ext[D] = 6;
    st[D]  = (std::size_t)g->em_s[3];
    return ndfield_t<D, 6>::wrap_strided(static_cast<real_t*>(p), ext, st);
  }

  template <Dimension D, FldsID::type F>
  void moment(const orc_grid* g, const orc_species* sp, int c1, int c2, int order, int smoothing,
              int use_weights, double inv_n0, double dx, void* bckp, int comp) {
    ntt::Particles<D, ntt::Coord::Cartesian> prt(1, "ref", sp->mass, sp->charge,
                                                 sp->npart > 0 ? (npart_t)sp->npart : 1, 0, 0,
                                                 ntt::ParticlePusher::BORIS, false,
                                                 ntt::RadiativeDrag::NONE,
                                                 ntt::EmissionType::NONE, 0, 0);
    fill<D>(prt, sp);
    std::vector<ncells_t> res { static_cast<ncells_t>(g->n1), static_cast<ncells_t>(g->n2) };
    boundaries_t<real_t>  ext { { ZERO, static_cast<real_t>(g->n1) * static_cast<real_t>(dx) },
                                { ZERO, static_cast<real_t>(g->n2) * static_cast<real_t>(dx) } };
    boundaries_t<FldsBC>  bcs { { FldsBC::PERIODIC, FldsBC::PERIODIC },
                                { FldsBC::PERIODIC, FldsBC::PERIODIC } };
    if constexpr (D == Dim::_3D) {
      res.push_back(static_cast<ncells_t>(g->n3));
      ext.push_back({ ZERO, static_cast<real_t>(g->n3) * static_cast<real_t>(dx) });
      bcs.push_back({ FldsBC::PERIODIC, FldsBC::PERIODIC });
    }
    const metric::Minkowski<D> metric(res, ext);
    auto                       buffer = wrap_em<D>(g, bckp);
    auto                       scatter = Kokkos::Experimental::create_scatter_view(buffer);
    std::vector<uint8_t>       comps;
    if (c1 > 0 || c2 > 0) {
      comps.push_back(static_cast<uint8_t>(c1));
      if (c2 > 0 || F == FldsID::T) {
        comps.push_back(static_cast<uint8_t>(c2));
      }
    }
    Kokkos::shim::g_serial = true;
    Kokkos::parallel_for("ComputeMoments", prt.rangeActiveParticles(),
                         kernel::ParticleMoments_kernel<SimEngine::SRPIC, metric::Minkowski<D>, F, 6>(
                           comps, scatter, static_cast<idx_t>(comp), prt, use_weights != 0, metric,
                           bcs, static_cast<ncells_t>(g->n2), static_cast<real_t>(inv_n0),
                           static_cast<uint8_t>(order),
                           static_cast<OutputSmoothingTypeFlag>(smoothing)));
    Kokkos::Experimental::contribute(buffer, scatter);
    Kokkos::shim::g_serial = false;
  }

  template <Dimension D>
  int moment_by_id(const orc_grid* g, const orc_species* sp, int id, int c1, int c2, int order,
                   int smoothing, int use_weights, double inv_n0, double dx, void* bckp,
                   int comp) {
    switch (id) {
      case 0: moment<D, FldsID::Rho>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      case 1: moment<D, FldsID::Charge>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      case 2: moment<D, FldsID::N>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      case 3: moment<D, FldsID::Nppc>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      case 4: moment<D, FldsID::T>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      case 5: moment<D, FldsID::V>(g, sp, c1, c2, order, smoothing, use_weights, inv_n0, dx, bckp, comp); break;
      default: return -1;
    }
    return 0;
  }

} // namespace

extern "C" {

// ComputeMoments for one species into component `comp` of a 6-component
// buffer with the oracle's em strides (added to what it holds); ids as
// orc_output_moment: 0 Rho, 1 Charge, 2 N, 3 Nppc, 4 T (c1, c2), 5 V (c1);
// smoothing 1 const, 2 spline
int ref_output_moment(const orc_grid* g, const orc_species* sp, int id, int c1, int c2, int order,
                      int smoothing, int use_weights, double inv_n0, double dx, void* bckp,
                      int comp) {
  if (g->ng != (int)N_GHOSTS) {
    return -2;
  }
  if (g->dim == 2) {
    return moment_by_id<Dim::_2D>(g, sp, id, c1, c2, order, smoothing, use_weights, inv_n0, dx,
                                  bckp, comp);
  }
  if (g->dim == 3) {
    return moment_by_id<Dim::_3D>(g, sp, id, c1, c2, order, smoothing, use_weights, inv_n0, dx,
                                  bckp, comp);
  }
  return -1;
}

// the species after RemoveDead (when remove_dead) and SortSpatially; returns
// the new particle count (-1 for an unsupported dimension). The payloads are
// row-major (particle, column) arrays, pld_i of npart_t (uint32).
std::int64_t ref_sort(const orc_grid* g, orc_species* sp, int remove_dead, void* pld_r,
                      int npld_r, std::uint32_t* pld_i, int npld_i) {
  if (g->dim == 2) {
    return sort_species<Dim::_2D>(g, sp, remove_dead, static_cast<real_t*>(pld_r), npld_r, pld_i,
                                  npld_i);
  }
  if (g->dim == 3) {
    return sort_species<Dim::_3D>(g, sp, remove_dead, static_cast<real_t*>(pld_r), npld_r, pld_i,
                                  npld_i);
  }
  return -1;
}

} // extern "C"
