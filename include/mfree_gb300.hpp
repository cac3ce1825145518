/*
 * mfree_gb300.hpp -- header-only C++14 facade over the C ABI (mfree_gb300.h) that keeps
 * the reference's scenario-code shape:
 *
 *   reference (rings.cpp:598-617)                      facade
 *   body<particle_monaghan> b(p, n, sim_data, dt);      mf::body b = ctx.add_body(p, n, sim_data, dt);
 *   b.set_boundary(new boundary<..>(convex_hull(..)));  b.set_boundary(mf::convex_hull(x, y, n));
 *   b.add_action(&material_eos);                        b.add_action(mf::material_eos);
 *   bc.add_boundary_condition(idx, &pull);              b.add_boundary_condition(idx, MF_BC_PULL, v);
 *   for (...) { b.step(); ... contact(...); }           ctx.step();   (all bodies, contact in main()'s order)
 *   b.get_particles()[i]->x                             b.get_state().x[i]
 *
 * Errors become mf::error (status + mf_last_error text) instead of the reference's
 * asserts and FP traps.  The context owns the device memory; copies are disabled,
 * moves allowed.
 */
#ifndef MFREE_GB300_HPP
#define MFREE_GB300_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mfree_gb300.h"

namespace mf {

// the reference's action functions, by name (body<T>::add_action(&name))
enum action : int32_t {
	riemann_update_integration_weights = MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS,
	material_eos = MF_MATERIAL_EOS,
	correctors_mghn_artificial_stress = MF_CORRECTORS_MGHN_ARTIFICIAL_STRESS,
	derive_stress_monaghan = MF_DERIVE_STRESS_MONAGHAN,
	derive_velocity = MF_DERIVE_VELOCITY,
	correctors_mghn_artificial_viscosity = MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
	correctors_xsph = MF_CORRECTORS_XSPH,
	material_stress_rate_jaumann = MF_MATERIAL_STRESS_RATE_JAUMANN,
	contmech_continuity = MF_CONTMECH_CONTINUITY,
	contmech_momentum_ul = MF_CONTMECH_MOMENTUM_UL,
	contmech_advection = MF_CONTMECH_ADVECTION,
	derive_displacement = MF_DERIVE_DISPLACEMENT,
	material_compute_stress_green_stvenant = MF_MATERIAL_COMPUTE_STRESS_GREEN_STVENANT,
	contmech_cauchy_to_nominal = MF_CONTMECH_CAUCHY_TO_NOMINAL,
	derive_stress_tl = MF_DERIVE_STRESS_TL,
	contmech_momentum_tl = MF_CONTMECH_MOMENTUM_TL,
	derive_velocity_tl = MF_DERIVE_VELOCITY_TL,
	contmech_velocity_gradient_tl = MF_CONTMECH_VELOCITY_GRADIENT_TL,
	derive_displacement_weak = MF_DERIVE_DISPLACEMENT_WEAK,
	derive_velocity_tl_weak = MF_DERIVE_VELOCITY_TL_WEAK,
	contmech_velocity_gradient_tl_gp = MF_CONTMECH_VELOCITY_GRADIENT_TL_GP,
	contmech_continuity_gp = MF_CONTMECH_CONTINUITY_GP,
	material_eos_gp = MF_MATERIAL_EOS_GP,
	material_stress_rate_jaumann_gp = MF_MATERIAL_STRESS_RATE_JAUMANN_GP,
	contmech_cauchy_to_nominal_gp = MF_CONTMECH_CAUCHY_TO_NOMINAL_GP,
	derive_stress_weak_tl = MF_DERIVE_STRESS_WEAK_TL,
	contmech_momentum_tl_weak = MF_CONTMECH_MOMENTUM_TL_WEAK,
	corotational_anisotropy_tensor = MF_COROTATIONAL_ANISOTROPY_TENSOR,
	derive_displacement_corotational = MF_DERIVE_DISPLACEMENT_COROTATIONAL,
	material_compute_stress_cauchy_green = MF_MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN,
	derive_stress_corotational = MF_DERIVE_STRESS_COROTATIONAL,
	godunov_continuity = MF_GODUNOV_CONTINUITY,
	godunov_momentum = MF_GODUNOV_MOMENTUM,
	potential_comp_elastic_potential = MF_POTENTIAL_COMP_ELASTIC_POTENTIAL
};

class error : public std::runtime_error {
public:
	error(mf_status s, const std::string& what) : std::runtime_error(what), status(s) {}
	mf_status status;
};

inline void check(mf_status s, const mf_ctx* ctx, const char* call) {
	if (s == MF_OK) return;
	std::string msg = std::string(call) + ": " + mf_status_string(s);
	const char* detail = ctx ? mf_last_error(ctx) : nullptr;
	if (detail && *detail) msg += std::string(" (") + detail + ")";
	throw error(s, msg);
}

// convex_hull(particles, n) (convex_hull.h:62-95): hull indices, tour order
inline std::vector<uint32_t> convex_hull(const double* x, const double* y, uint32_t n) {
	std::vector<uint32_t> idx(n);
	uint32_t nb = 0;
	check(mf_convex_hull(x, y, n, idx.data(), &nb), nullptr, "mf_convex_hull");
	idx.resize(nb);
	return idx;
}

// A body's state after a step, host SoA (the fields of particle.h:42-47 that evolve).
struct state {
	std::vector<double> x, y, vx, vy, rho, Sxx, Sxy, Syy, fcx, fcy;
};

class context;

// Handle on one body of a context (body<T> of the reference).
class body {
public:
	body() = default;
	body(mf_ctx* ctx, int32_t id) : ctx_(ctx), id_(id) {}
	int32_t id() const { return id_; }

	void add_action(action a) { check(mf_add_action(ctx_, id_, a), ctx_, "mf_add_action"); }
	void set_boundary(const std::vector<uint32_t>& idx) {
		check(mf_set_boundary(ctx_, id_, idx.data(), (uint32_t)idx.size()), ctx_, "mf_set_boundary");
	}
	void add_boundary_condition(const std::vector<uint32_t>& idx, mf_bc_kind kind, double v) {
		check(mf_add_boundary_condition(ctx_, id_, idx.data(), (uint32_t)idx.size(), kind, v), ctx_,
		      "mf_add_boundary_condition");
	}
	// particle_tl_weak bodies: element_map_rectangle(ex, ey) and the Gauss points' h and rho
	void set_gauss_mesh(uint32_t ex, uint32_t ey, double gp_h, double gp_rho) {
		check(mf_set_gauss_mesh(ctx_, id_, ex, ey, gp_h, gp_rho), ctx_, "mf_set_gauss_mesh");
	}
	// weak bodies on an explicit element map (gauss_int(elements, order)): quads holds
	// ll, lr, tr, tl per element; MF_SHAPE_ELEMENT for the *_fem set-ups
	void set_elements(const std::vector<uint32_t>& quads, uint32_t order, int32_t shape, double gp_h = 0.,
	                  double gp_rho = 0.) {
		check(mf_set_elements(ctx_, id_, quads.data(), (uint32_t)(quads.size() / 4), order, shape, gp_h, gp_rho), ctx_,
		      "mf_set_elements");
	}
	// particle_ul_weak: the stress points (the particles' 13 fields)
	void set_stress_points(const mf_particles& sp, uint32_t n) {
		check(mf_set_stress_points(ctx_, id_, &sp, n), ctx_, "mf_set_stress_points");
	}
	// particle_tl_weak: the Gauss points' position, h and rho as the set-up left them
	void set_gauss_points(const std::vector<double>& x, const std::vector<double>& y, const std::vector<double>& h,
	                      const std::vector<double>& rho) {
		check(mf_set_gauss_points(ctx_, id_, x.data(), y.data(), h.data(), rho.data(), (uint32_t)x.size()), ctx_,
		      "mf_set_gauss_points");
	}
	uint32_t get_num_part() const {
		uint32_t n = 0;
		check(mf_num_particles(ctx_, id_, &n), ctx_, "mf_num_particles");
		return n;
	}
	double get_time() const {
		double t = 0.;
		check(mf_get_time(ctx_, id_, &t), ctx_, "mf_get_time");
		return t;
	}
	state get_state() const {
		const uint32_t n = get_num_part();
		state s;
		std::vector<double>* f[10] = {&s.x, &s.y, &s.vx, &s.vy, &s.rho, &s.Sxx, &s.Sxy, &s.Syy, &s.fcx, &s.fcy};
		for (auto* v : f) v->resize(n);
		mf_state out = {s.x.data(), s.y.data(), s.vx.data(), s.vy.data(), s.rho.data(),
		                s.Sxx.data(), s.Sxy.data(), s.Syy.data(), s.fcx.data(), s.fcy.data()};
		check(mf_get_state(ctx_, id_, &out), ctx_, "mf_get_state");
		return s;
	}
	void set_state(const mf_particles& p) { check(mf_set_state(ctx_, id_, &p), ctx_, "mf_set_state"); }

private:
	mf_ctx* ctx_ = nullptr;
	int32_t id_ = -1;
};

// One simulation (or an ensemble of independent ones, by group) on one GPU.
class context {
public:
	explicit context(mf_method method, mf_precision precision = MF_PREC_FP64_STRICT, int32_t device = 0,
	                 bool contact = false, double nbh_eps = 1e-6, double nbh_h = 0., uint32_t max_nbh = 200,
	                 bool graph = false) {
		mf_config cfg = {method, precision, device, max_nbh, nbh_eps, nbh_h, contact ? 1 : 0, graph ? 1 : 0};
		check(mf_create(&cfg, &ctx_), nullptr, "mf_create");
	}
	~context() {
		if (ctx_) mf_destroy(ctx_);
	}
	context(const context&) = delete;
	context& operator=(const context&) = delete;
	context(context&& o) noexcept : ctx_(o.ctx_) { o.ctx_ = nullptr; }
	context& operator=(context&& o) noexcept {
		std::swap(ctx_, o.ctx_);
		return *this;
	}

	// body(particles, n, simulation_data, dt) (body.h:228-233); group: contact partners
	body add_body(const mf_particles& p, uint32_t n, const mf_sim_data& sd, double dt, int32_t group = 0) {
		int32_t id = -1;
		check(mf_add_body(ctx_, &p, n, &sd, dt, group, &id), ctx_, "mf_add_body");
		return body(ctx_, id);
	}
	// nsteps of main()'s loop (mfree_iwf.cpp:84-97) over every body
	void step(int32_t nsteps = 1) { check(mf_step(ctx_, nsteps), ctx_, "mf_step"); }
	void synchronize() { check(mf_synchronize(ctx_), ctx_, "mf_synchronize"); }
	std::string autotune(int32_t trial_steps = 3) {
		char rep[1024] = {0};
		check(mf_autotune(ctx_, trial_steps, rep, sizeof rep), ctx_, "mf_autotune");
		return rep;
	}
	mf_ctx* raw() { return ctx_; }

private:
	mf_ctx* ctx_ = nullptr;
};

}  // namespace mf

#endif
