// mpm_ops.cuh -- launch wrappers that bind the kernels of one arithmetic form
// into a StepOps table (included once per form).
#pragma once

#include "mpm_kernels.cuh"

namespace mpm {

inline unsigned grid_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

template <class P>
struct Ops {
  static St<P>& S(void* st) { return *reinterpret_cast<St<P>*>(st); }

  static void begin_step(void* st, const Geometry&, cudaStream_t s) {
    prof_begin(K_BEGIN, s);
    k_begin_step<<<1, 1, 0, s>>>(S(st).sc);
    prof_end(K_BEGIN, s);
  }
  static void locate(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_LOCATE, s);
    k_locate<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g, g.shape == 3 ? g.ncell : (int)g.nnt);
    prof_end(K_LOCATE, s);
  }
  static void node_offsets(void*, const Geometry&, long long, cudaStream_t) {}
  static void p2g_mass(void* st, const Geometry& g, int bc, int vel, cudaStream_t s) {
    prof_begin(K_P2G_MASS, s);
    if (g.shape == 3) {
      k_sg_cell_mass<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_sg_node_mass<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g, bc, vel);
    } else {
      k_p2g_mass<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g, bc, vel);
    }
    prof_end(K_P2G_MASS, s);
  }
  static void node_velocity(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_NODE_VEL, s);
    k_node_velocity<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g);
    prof_end(K_NODE_VEL, s);
  }
  static void apply_bc(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_BC, s);
    k_apply_bc<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g);
    prof_end(K_BC, s);
  }
  static void stress(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_STRESS, s);
    if (g.shape == 3) k_sg_cell_gradient<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
    k_stress<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    prof_end(K_STRESS, s);
  }
  static void depeff_apply(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_DEPEFF, s);
    k_depeff_apply<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    k_depeff_carry<P><<<1, 1, 0, s>>>(S(st), g);
    prof_end(K_DEPEFF, s);
  }
  static void force_prep(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_FORCE_PREP, s);
    k_force_prep<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    prof_end(K_FORCE_PREP, s);
  }
  static void p2g_force(void* st, const Geometry& g, int integ, cudaStream_t s) {
    prof_begin(K_P2G_FORCE, s);
    if (g.shape == 3) {
      k_sg_cell_force<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_sg_node_force<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g, integ);
    } else {
      k_p2g_force<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g, integ);
    }
    prof_end(K_P2G_FORCE, s);
  }
  static void integrate(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_INTEGRATE, s);
    k_integrate<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g);
    prof_end(K_INTEGRATE, s);
  }
  static void position(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_POSITION, s);
    if (g.shape == 3) k_sg_cell_velocity<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
    k_position<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    prof_end(K_POSITION, s);
  }
  static void p2g_momentum(void* st, const Geometry& g, int vel, cudaStream_t s) {
    prof_begin(K_P2G_MOM, s);
    if (g.shape == 3) {
      k_sg_cell_momentum<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_sg_node_momentum<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g, vel);
    } else {
      k_p2g_momentum<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g, vel);
    }
    prof_end(K_P2G_MOM, s);
  }
  static void reduce(void* st, const Geometry& g, int mode, int nblocks, cudaStream_t s) {
    prof_begin(K_REDUCE, s);
    k_reduce<P><<<nblocks, kBlock, 0, s>>>(S(st), g, mode);
    prof_end(K_REDUCE, s);
  }
  static void dr_damping(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_DR, s);
    k_dr_damping<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    k_dr_finish<<<1, 1, 0, s>>>(S(st).sc);
    prof_end(K_DR, s);
  }

  static void fixed_locate(void* st, const Geometry& g, int with_comp, cudaStream_t s) {
    prof_begin(K_LOCATE, s);
    k_fixed_locate<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g, g.shape == 3 ? g.ncell : (int)g.nnt, with_comp);
    prof_end(K_LOCATE, s);
  }
  static void tl_initial(void* st, const Geometry& g, cudaStream_t s) {
    k_tl_initial<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
  }
  static void tl_momentum(void* st, const Geometry& g, int vel, cudaStream_t s) {
    prof_begin(K_P2G_MASS, s);
    if (g.shape == 3) {
      k_sg_cell_momentum<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_tl_sg_node_momentum<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g, vel);
    } else {
      k_p2g_momentum<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g, vel);
    }
    prof_end(K_P2G_MASS, s);
  }
  static void tl_stress(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_STRESS, s);
    if (g.shape == 3) k_sg_cell_gradient<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
    k_tl_stress<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    prof_end(K_STRESS, s);
  }
  static void tl_force(void* st, const Geometry& g, int integ, cudaStream_t s) {
    prof_begin(K_P2G_FORCE, s);
    if (g.shape == 3) {
      k_tl_sg_cell_force<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_tl_sg_node_force<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g, integ);
    } else {
      k_tl_p2g_force<P><<<grid_for(g.nnt), kBlock, 0, s>>>(S(st), g, integ);
    }
    prof_end(K_P2G_FORCE, s);
  }
  static void smooth(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_SMOOTH, s);
    if (g.shape == 3) {
      k_smooth_cell<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
      k_smooth_sg_node<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g);
      k_smooth_sg_back<P><<<grid_for(g.ncell), kBlock, 0, s>>>(S(st), g);
    } else {
      k_smooth_node<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g);
    }
    k_smooth_g2p<P><<<grid_for(g.np), kBlock, 0, s>>>(S(st), g);
    prof_end(K_SMOOTH, s);
  }

  static void contact(void* st, const Geometry& g, cudaStream_t s) {
    prof_begin(K_CONTACT, s);
    k_contact<P><<<grid_for(g.nn), kBlock, 0, s>>>(S(st), g);
    k_contact_sum<P><<<1, kBlock, 0, s>>>(S(st), g);
    prof_end(K_CONTACT, s);
  }

  static StepOps table(const char* name) {
    StepOps o;
    o.name = name;
    o.bulk_size = sizeof(typename P::B);
    o.real_size = sizeof(typename P::R);
    o.begin_step = begin_step;
    o.locate = locate;
    o.node_offsets = node_offsets;
    o.p2g_mass = p2g_mass;
    o.node_velocity = node_velocity;
    o.apply_bc = apply_bc;
    o.stress = stress;
    o.depeff_apply = depeff_apply;
    o.force_prep = force_prep;
    o.p2g_force = p2g_force;
    o.integrate = integrate;
    o.position = position;
    o.p2g_momentum = p2g_momentum;
    o.reduce = reduce;
    o.dr_damping = dr_damping;
    o.fixed_locate = fixed_locate;
    o.tl_initial = tl_initial;
    o.tl_momentum = tl_momentum;
    o.tl_stress = tl_stress;
    o.tl_force = tl_force;
    o.smooth = smooth;
    o.contact = contact;
    return o;
  }
};

}  // namespace mpm
