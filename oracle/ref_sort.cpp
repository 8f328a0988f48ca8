// The reference's own particle sort on the host Kokkos shim (TEST
// INFRASTRUCTURE ONLY): Particles::RemoveDead and Particles::SortSpatially
// (src/framework/containers/particles_sort.cpp:103-253), run on a species
// copied into an ntt::Particles<D, Cartesian> container (particles.cpp), then
// copied back in the new order. Built with the reference's container and grid
// sources by oracle/build_ref.py; adds no logic of its own.
//
// The shim runs these calls serially in index order (Kokkos::shim::g_serial):
// RemoveDead hands out the alive slots with an atomic counter and BinSort
// fills each bin in element order, which on a serial host is the particles'
// original order. Kokkos leaves both orders to the backend.
#include "enums.h"
#include "global.h"

#include "arch/kokkos_aliases.h"

#include "framework/containers/particles.h"
#include "framework/domain/grid.h"

#include "srpic_oracle.h"

#include <cstdint>
#include <vector>

namespace {

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

} // namespace

extern "C" {

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
