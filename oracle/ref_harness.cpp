// Test infrastructure: drives the reference's own, unmodified sources (compiled
// out of tree by oracle/build_ref.sh against the project-written GLM subset) so
// that the CPU oracle restatement and the golden fixtures can be pinned to the
// reference itself.  Never shipped, never part of the product.
//
//   ref_harness run CASE RESULT
//       builds the bodies of CASE with the reference's particle classes, body<T>,
//       action functions, find_neighbors/precomp_* set-up and contact, runs the
//       step loop of main() (mfree_iwf.cpp:84-97) and writes RESULT.
//   ref_harness scenario NAME NBOX NSTEPS CASE_OUT RESULT
//       runs one of the reference's own scenario builders (rings_monaghan,
//       rings_monaghan_contact, rings_tl_contact, tensile_tl, tensile_tl_weak)
//       unchanged, writes its initial state as CASE_OUT (so the restatement can
//       replay it) and the run as RESULT.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "body.h"
#include "contact.h"
#include "particle.h"
#include "benchmarks/rings.h"
#include "benchmarks/tensile.h"
#include "benchmarks/rotation.h"
#include "benchmarks/utils.h"
#include "interpolation.h"

#include "vtk_writer.h"

#include <unistd.h>

#include "mfcase.h"

using namespace mfcase;

namespace {

// neighbour lists of the first derivative evaluation, by particle idx
std::vector<std::vector<std::vector<unsigned>>> g_nbh;
int g_cur_body = 0;
std::vector<bool> g_recorded;

template <typename T>
void record_first_nbh(body<T>& b) {
	if (g_recorded[g_cur_body]) return;
	g_recorded[g_cur_body] = true;
	T** p = b.get_cur_particles();
	unsigned n = b.get_num_part();
	auto& L = g_nbh[g_cur_body];
	L.assign(n, {});
	for (unsigned i = 0; i < n; i++)
		for (unsigned j = 0; j < p[i]->num_nbh; j++) L[p[i]->idx].push_back(p[p[i]->nbh[j]]->idx);
}

// The stress points of a particle_ul_weak body as its builder made them: the body
// keeps them private, so this action (run after the others) copies them at the first
// derivative evaluation, where the stage copies still hold the built values except
// h (set by the neighbour search) and the velocity (set by
// interpolation_interpolate_velocity); neither is an input of the method, both are
// written as zero.
std::vector<BodyIn> g_gp;
std::vector<bool> g_gp_done;
template <typename T>
void capture_gp(body<T>& b) {
	if (g_gp_done[g_cur_body]) return;
	g_gp_done[g_cur_body] = true;
	BodyIn& g = g_gp[g_cur_body];
	T** q = b.get_cur_quad_points();
	g.n = b.get_num_quad_points();
	for (int k = 0; k < NIN; k++) g.a[k].resize(g.n);
	for (unsigned i = 0; i < g.n; i++) {
		double f[NIN] = {q[i]->x, q[i]->y, q[i]->X, q[i]->Y, q[i]->m, q[i]->rho, 0., q[i]->quad_weight,
		                 0., 0., q[i]->Sxx, q[i]->Sxy, q[i]->Syy};
		for (int k = 0; k < NIN; k++) g.a[k][i] = f[k];
	}
}

// The Gauss points of a particle_tl_weak body as its set-up left them (the body keeps
// them private): copied at the first derivative evaluation, where nothing has changed
// their position, h or density yet.
template <typename T>
void capture_gp_tl(body<T>& b) {
	if (g_gp_done[g_cur_body]) return;
	g_gp_done[g_cur_body] = true;
	BodyIn& g = g_gp[g_cur_body];
	T** q = b.get_cur_quad_points();
	g.n = b.get_num_quad_points();
	for (int k = 0; k < NIN; k++) g.a[k].resize(g.n);
	for (unsigned i = 0; i < g.n; i++) {
		double f[NIN] = {q[i]->x, q[i]->y, q[i]->X, q[i]->Y, q[i]->m, q[i]->rho, q[i]->h, q[i]->quad_weight,
		                 q[i]->vx, q[i]->vy, q[i]->Sxx, q[i]->Sxy, q[i]->Syy};
		for (int k = 0; k < NIN; k++) g.a[k][i] = f[k];
	}
}

template <typename T>
void record_fixed_nbh(T** p, unsigned n, int b) {
	auto& L = g_nbh[b];
	L.assign(n, {});
	for (unsigned i = 0; i < n; i++)
		for (unsigned j = 0; j < p[i]->num_nbh; j++) L[p[i]->idx].push_back(p[p[i]->nbh[j]]->idx);
	g_recorded[b] = true;
}

typedef void (*UlAct)(body<particle_monaghan>&);
typedef void (*TlAct)(body<particle_tl>&);
typedef void (*WkAct)(body<particle_tl_weak>&);
typedef void (*CrAct)(body<particle_corotational>&);
typedef void (*PtAct)(body<particle_potential>&);
typedef void (*UwAct)(body<particle_ul_weak>&);

UlAct ul_action(uint32_t a) {
	typedef particle_monaghan T;
	switch (a) {
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS: return &riemann_update_integration_weights<T>;
	case MATERIAL_EOS: return &material_eos<T>;
	case CORRECTORS_MGHN_ARTIFICIAL_STRESS: return &correctors_mghn_artificial_stress<T>;
	case DERIVE_STRESS_MONAGHAN: return &derive_stress_monaghan<T>;
	case DERIVE_VELOCITY: return &derive_velocity<T>;
	case CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY: return &correctors_mghn_artificial_viscosity<T>;
	case CORRECTORS_XSPH: return &correctors_xsph<T>;
	case MATERIAL_STRESS_RATE_JAUMANN: return &material_stress_rate_jaumann<T>;
	case CONTMECH_CONTINUITY: return &contmech_continuity<T>;
	case CONTMECH_MOMENTUM_UL: return &contmech_momentum_ul<T>;
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case GODUNOV_CONTINUITY: return &godunov_continuity<T>;
	case GODUNOV_MOMENTUM: return &godunov_momentum<T>;
	}
	return nullptr;
}
PtAct pt_action(uint32_t a) {
	typedef particle_potential T;
	switch (a) {
	case CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY: return &correctors_mghn_artificial_viscosity<T>;
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case DERIVE_DISPLACEMENT: return &derive_displacement<T>;
	case MATERIAL_COMPUTE_STRESS_GREEN_STVENANT: return &material_compute_stress_green_stvenant<T>;
	case POTENTIAL_COMP_ELASTIC_POTENTIAL: return &potential_comp_elastic_potential<T>;
	}
	return nullptr;
}
UwAct uw_action(uint32_t a) {
	typedef particle_ul_weak T;
	switch (a) {
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS: return &riemann_update_integration_weights<T>;
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP: return &riemann_update_integration_weights_gp<T>;
	case MATERIAL_EOS_GP: return &material_eos_gp<T>;
	case DERIVE_STRESS_WEAK_UL: return &derive_stress_weak_ul<T>;
	case DERIVE_VELOCITY_WEAK: return &derive_velocity_weak<T>;
	case DERIVE_VELOCITY: return &derive_velocity<T>;
	case MATERIAL_STRESS_RATE_JAUMANN_GP: return &material_stress_rate_jaumann_gp<T>;
	case CONTMECH_MOMENTUM_UL: return &contmech_momentum_ul<T>;
	case CONTMECH_MOMENTUM_UL_WEAK: return &contmech_momentum_ul_weak<T>;
	case CONTMECH_CONTINUITY: return &contmech_continuity<T>;
	case CONTMECH_CONTINUITY_GP: return &contmech_continuity_gp<T>;
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case INTERPOLATION_INTERPOLATE_VELOCITY: return &interpolation_interpolate_velocity<T>;
	case CONTMECH_ADVECTION_GP: return &contmech_advection_gp<T>;
	}
	return nullptr;
}
TlAct tl_action(uint32_t a) {
	typedef particle_tl T;
	switch (a) {
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS: return &riemann_update_integration_weights<T>;
	case MATERIAL_EOS: return &material_eos<T>;
	case DERIVE_VELOCITY: return &derive_velocity<T>;
	case CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY: return &correctors_mghn_artificial_viscosity<T>;
	case CORRECTORS_XSPH: return &correctors_xsph<T>;
	case MATERIAL_STRESS_RATE_JAUMANN: return &material_stress_rate_jaumann<T>;
	case CONTMECH_CONTINUITY: return &contmech_continuity<T>;
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case DERIVE_DISPLACEMENT: return &derive_displacement<T>;
	case MATERIAL_COMPUTE_STRESS_GREEN_STVENANT: return &material_compute_stress_green_stvenant<T>;
	case CONTMECH_CAUCHY_TO_NOMINAL: return &contmech_cauchy_to_nominal<T>;
	case DERIVE_STRESS_TL: return &derive_stress_tl<T>;
	case CONTMECH_MOMENTUM_TL: return &contmech_momentum_tl<T>;
	case DERIVE_VELOCITY_TL: return &derive_velocity_tl<T>;
	case CONTMECH_VELOCITY_GRADIENT_TL: return &contmech_velocity_gradient_tl<T>;
	}
	return nullptr;
}
CrAct cr_action(uint32_t a) {
	typedef particle_corotational T;
	switch (a) {
	case CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY: return &correctors_mghn_artificial_viscosity<T>;
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case CONTMECH_CAUCHY_TO_NOMINAL: return &contmech_cauchy_to_nominal<T>;
	case COROTATIONAL_ANISOTROPY_TENSOR: return &corotational_anisotropy_tensor<T>;
	case DERIVE_DISPLACEMENT_COROTATIONAL: return &derive_displacement_corotational<T>;
	case MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN: return &material_compute_stress_cauchy_green<T>;
	case DERIVE_STRESS_COROTATIONAL: return &derive_stress_corotational<T>;
	}
	return nullptr;
}
WkAct wk_action(uint32_t a) {
	typedef particle_tl_weak T;
	switch (a) {
	case CONTMECH_ADVECTION: return &contmech_advection<T>;
	case DERIVE_DISPLACEMENT_WEAK: return &derive_displacement_weak<T>;
	case DERIVE_VELOCITY_TL_WEAK: return &derive_velocity_tl_weak<T>;
	case CONTMECH_VELOCITY_GRADIENT_TL_GP: return &contmech_velocity_gradient_tl_gp<T>;
	case CONTMECH_CONTINUITY_GP: return &contmech_continuity_gp<T>;
	case MATERIAL_EOS_GP: return &material_eos_gp<T>;
	case MATERIAL_STRESS_RATE_JAUMANN_GP: return &material_stress_rate_jaumann_gp<T>;
	case CONTMECH_CAUCHY_TO_NOMINAL_GP: return &contmech_cauchy_to_nominal_gp<T>;
	case DERIVE_STRESS_WEAK_TL: return &derive_stress_weak_tl<T>;
	case CONTMECH_MOMENTUM_TL_WEAK: return &contmech_momentum_tl_weak<T>;
	}
	return nullptr;
}

// --- pull boundary conditions of tensile.cpp:20-42 with a case-given speed.  A
// boundary_conditions<T> functor is a plain function pointer, so each speed in
// use gets a slot in a small table.
double g_bc_speed[8];
template <typename T, int K>
void pull_bc(T* p) {
	double v = g_bc_speed[K];
	p->x = p->X + v * simulation_time::getInstance().get_time();
	p->y = p->Y;
	p->vx = v;
	p->vy = 0.;
	p->vx_t = 0.;
	p->vy_t = 0.;
}
// the updated-Lagrangian form (tensile.cpp:44-66)
template <typename T, int K>
void vel_bc(T* p) {
	double v = g_bc_speed[K];
	p->x_t = v;
	p->y_t = 0.;
	p->vx = v;
	p->vy = 0.;
	p->vx_t = 0.;
	p->vy_t = 0.;
}
template <typename T>
void (*vel_fn(int k))(T*) {
	switch (k) {
	case 0: return &vel_bc<T, 0>;
	case 1: return &vel_bc<T, 1>;
	case 2: return &vel_bc<T, 2>;
	case 3: return &vel_bc<T, 3>;
	}
	return nullptr;
}
template <typename T>
void (*pull_fn(int k))(T*) {
	switch (k) {
	case 0: return &pull_bc<T, 0>;
	case 1: return &pull_bc<T, 1>;
	case 2: return &pull_bc<T, 2>;
	case 3: return &pull_bc<T, 3>;
	}
	return nullptr;
}

simulation_data make_sim_data(const Case& c) {
	physical_constants pc(c.nu, c.E, c.rho0);
	correction_constants cc(constants_monaghan(c.wdeltap, c.corr_exp, c.mghn_eps),
	                        constants_artificial_viscosity(c.alpha, c.beta, c.eta), c.xsph_eps, c.do_smooth != 0);
	return simulation_data(pc, cc);
}

template <typename T>
T** make_particles(const BodyIn& in) {
	T** p = new T*[in.n];
	for (unsigned i = 0; i < in.n; i++) {
		p[i] = new T(i);
		double* f[NIN] = {&p[i]->x, &p[i]->y, &p[i]->X, &p[i]->Y, &p[i]->m, &p[i]->rho, &p[i]->h, &p[i]->quad_weight,
		                  &p[i]->vx, &p[i]->vy, &p[i]->Sxx, &p[i]->Sxy, &p[i]->Syy};
		for (int a = 0; a < NIN; a++) *f[a] = in.a[a][i];
	}
	return p;
}

template <typename T>
boundary_conditions<T> make_bcs(const BodyIn& in, int& slot) {
	boundary_conditions<T> bc;
	for (const BC& b : in.bcs) {
		if ((b.kind != BC_PULL_TL && b.kind != BC_VELOCITY_UL) || slot >= 4) {
			fprintf(stderr, "unsupported boundary condition\n");
			exit(2);
		}
		g_bc_speed[slot] = b.v;
		bc.add_boundary_condition(b.idx, b.kind == BC_PULL_TL ? pull_fn<T>(slot) : vel_fn<T>(slot));
		slot++;
	}
	return bc;
}

void write_header(Writer& w, const Case& c) {
	w.raw("MFOUT1\0\0", 8);
	w.u32(c.nbodies);
	for (auto& b : c.bodies) w.u32(b.n);
}

template <typename T>
void dump(Writer& w, unsigned step, std::vector<body<T>>& bodies) {
	w.u32(1);
	w.u32(step);
	w.f64(simulation_time::getInstance().get_time());
	for (auto& b : bodies) {
		T** p = b.get_particles();
		unsigned n = b.get_num_part();
		for (int k = 0; k < NOUT; k++)
			for (unsigned i = 0; i < n; i++) {
				double v = 0.;
				switch (k) {
				case 0: v = p[i]->x; break;
				case 1: v = p[i]->y; break;
				case 2: v = p[i]->vx; break;
				case 3: v = p[i]->vy; break;
				case 4: v = p[i]->rho; break;
				case 5: v = p[i]->Sxx; break;
				case 6: v = p[i]->Sxy; break;
				case 7: v = p[i]->Syy; break;
				case 8: v = p[i]->fcx; break;
				case 9: v = p[i]->fcy; break;
				}
				w.f64(v);
			}
	}
}

// set by `run CASE RESULT VTKDIR`: also write the final state with vtk_writer_write
const char* g_vtk_dir = nullptr;

template <typename T>
void run_loop(Writer& w, const Case& c, std::vector<body<T>>& bodies) {
	double secs = 0.;
	for (unsigned s = 1; s <= c.nsteps; s++) {
		auto t0 = std::chrono::steady_clock::now();
		for (unsigned i = 0; i < bodies.size(); i++) {
			g_cur_body = (int)i;
			bodies[i].step();
			bodies[i].update_boundary();
		}
		if (c.contact)
			for (unsigned i = 0; i < bodies.size(); i++)
				for (unsigned j = 0; j < bodies.size(); j++)
					if (i != j) contact_apply_body_to_boundary(bodies[i], bodies[j]);
		secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
		if ((c.dump_every && s % c.dump_every == 0) || s == c.nsteps) dump(w, s, bodies);
	}
	if (c.nsteps == 0) dump(w, 0, bodies);
	if (g_vtk_dir) {
		// the reference's own writer: results/out_%06d.vtk below the given directory
		char cwd[4096];
		if (getcwd(cwd, sizeof cwd) && chdir(g_vtk_dir) == 0) {
			vtk_writer_write(bodies, c.nsteps);
			if (chdir(cwd) != 0) fprintf(stderr, "cannot return to %s\n", cwd);
		}
	}
	w.u32(2);
	for (unsigned b = 0; b < bodies.size(); b++) {
		auto& L = g_nbh[b];
		unsigned n = bodies[b].get_num_part();
		w.u32(n);
		for (unsigned i = 0; i < n; i++) w.u32(i < L.size() ? (uint32_t)L[i].size() : 0u);
		for (unsigned i = 0; i < n && i < L.size(); i++) w.raw(L[i].data(), L[i].size() * 4);
	}
	w.u32(3);
	w.f64(secs);
	w.u32(0);
}

template <typename T>
void attach_hull(body<T>& b, const std::vector<uint32_t>& hull) {
	if (hull.empty()) return;
	std::vector<unsigned int> idx(hull.begin(), hull.end());
	b.set_boundary(new boundary<T>(idx, b.get_particles()));
}

int run_case(const Case& c, const char* out) {
	Writer w(out);
	write_header(w, c);
	g_nbh.assign(c.nbodies, {});
	g_recorded.assign(c.nbodies, false);
	simulation_data sd = make_sim_data(c);
	int slot = 0;
	if (c.nbh_eps != 1e-6 && c.method != UL) {
		fprintf(stderr, "the reference's find_neighbors has a fixed 1e-6 epsilon\n");
		return 2;
	}
	if (c.method == UL) {
		if (c.nbh_eps != 1e-6) { fprintf(stderr, "the reference's grid has a fixed 1e-6 epsilon\n"); return 2; }
		typedef particle_monaghan T;
		std::vector<body<T>> bodies;
		for (const BodyIn& in : c.bodies) {
			T** p = make_particles<T>(in);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot)));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				UlAct f = ul_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for UL\n", a); return 2; }
				bodies[b].add_action(f);
			}
			bodies[b].add_action(&record_first_nbh<T>);
		}
		run_loop(w, c, bodies);
	} else if (c.method == TL) {
		typedef particle_tl T;
		std::vector<body<T>> bodies;
		for (unsigned b = 0; b < c.nbodies; b++) {
			const BodyIn& in = c.bodies[b];
			T** p = make_particles<T>(in);
			find_neighbors(p, in.n, c.nbh_h, distance_euclidian);
			precomp_randles_libersky<T>(p, in.n);
			record_fixed_nbh(p, in.n, (int)b);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot)));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				TlAct f = tl_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for TL\n", a); return 2; }
				bodies[b].add_action(f);
			}
		}
		run_loop(w, c, bodies);
	} else if (c.method == COROT) {
		typedef particle_corotational T;
		std::vector<body<T>> bodies;
		for (unsigned b = 0; b < c.nbodies; b++) {
			const BodyIn& in = c.bodies[b];
			T** p = make_particles<T>(in);
			find_neighbors(p, in.n, c.nbh_h, distance_euclidian);
			precomp_sph<T>(p, in.n);
			record_fixed_nbh(p, in.n, (int)b);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot)));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				CrAct f = cr_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for the corotational method\n", a); return 2; }
				bodies[b].add_action(f);
			}
		}
		run_loop(w, c, bodies);
	} else if (c.method == POTENTIAL) {
		typedef particle_potential T;
		std::vector<body<T>> bodies;
		for (unsigned b = 0; b < c.nbodies; b++) {
			const BodyIn& in = c.bodies[b];
			T** p = make_particles<T>(in);
			find_neighbors(p, in.n, c.nbh_h, distance_euclidian);
			precomp_randles_libersky_symmetric<T>(p, in.n);
			record_fixed_nbh(p, in.n, (int)b);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot)));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				PtAct f = pt_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for the potential method\n", a); return 2; }
				bodies[b].add_action(f);
			}
		}
		run_loop(w, c, bodies);
	} else if (c.method == UL_WEAK) {
		typedef particle_ul_weak T;
		std::vector<body<T>> bodies;
		for (unsigned b = 0; b < c.nbodies; b++) {
			const BodyIn& in = c.bodies[b];
			T** p = make_particles<T>(in);
			BodyIn gin;
			gin.n = in.ngp;
			for (int k = 0; k < NIN; k++) gin.a[k] = in.g[k];
			T** q = make_particles<T>(gin);
			if (in.ex == 1) {
				// a gauss_int in place of the ellipse (body.h:91-99, the *_ul_fem set-ups)
				std::vector<element> elements;
				for (size_t e = 0; e + 3 < in.quads.size(); e += 4)
					elements.push_back(element(in.quads[e], in.quads[e + 1], in.quads[e + 2], in.quads[e + 3]));
				gauss_int* gi = new gauss_int(elements, in.order);
				bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot), q, in.ngp, gi));
				continue;
			}
			find_neighbors(p, in.n, c.nbh_h, distance_manhattan);
			find_neighbors(p, in.n, q, in.ngp, c.nbh_h, distance_manhattan);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot), q, in.ngp));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				UwAct f = uw_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for UL_WEAK\n", a); return 2; }
				bodies[b].add_action(f);
			}
			bodies[b].add_action(&record_first_nbh<T>);
		}
		run_loop(w, c, bodies);
	} else if (c.method == TL_WEAK) {
		typedef particle_tl_weak T;
		std::vector<body<T>> bodies;
		for (unsigned b = 0; b < c.nbodies; b++) {
			const BodyIn& in = c.bodies[b];
			T** p = make_particles<T>(in);
			std::vector<element> elements;
			if (in.ex) {
				elements = element_map_rectangle(in.ex, in.ey);
			} else {
				for (size_t e = 0; e + 3 < in.quads.size(); e += 4)
					elements.push_back(element(in.quads[e], in.quads[e + 1], in.quads[e + 2], in.quads[e + 3]));
			}
			const unsigned order = in.ex ? 2 : in.order;
			unsigned num_gp = order * order * elements.size();
			T** gp = new T*[num_gp];
			for (unsigned i = 0; i < num_gp; i++) gp[i] = new T(i);
			gauss_int gi(elements, order);
			// the set-ups place the Gauss points before they move any body: from X
			std::vector<double> sx(in.n), sy(in.n);
			for (unsigned i = 0; i < in.n; i++) { sx[i] = p[i]->x; sy[i] = p[i]->y; p[i]->x = p[i]->X; p[i]->y = p[i]->Y; }
			gi.update_gauss_points(p, gp);
			for (unsigned i = 0; i < in.n; i++) { p[i]->x = sx[i]; p[i]->y = sy[i]; }
			const bool given = !in.ex && in.ngp == num_gp;
			for (unsigned i = 0; i < num_gp; i++) {
				gp[i]->h = given ? in.g[6][i] : c.gp_h;
				gp[i]->rho = given ? in.g[5][i] : c.gp_rho;
				if (given) { gp[i]->x = in.g[0][i]; gp[i]->y = in.g[1][i]; }
			}
			if (in.ex || in.shape == SHAPE_RKPM) {
				find_neighbors(p, in.n, c.nbh_h, distance_euclidian);
				find_neighbors(p, in.n, gp, num_gp, c.nbh_h, distance_euclidian);
				precomp_rkpm<T>(p, gp, num_gp);
				precomp_rkpm<T>(p, in.n);
			}
			record_fixed_nbh(p, in.n, (int)b);
			bodies.push_back(body<T>(p, in.n, sd, c.dt, make_bcs<T>(in, slot), gp, num_gp));
		}
		for (unsigned b = 0; b < c.nbodies; b++) {
			attach_hull(bodies[b], c.bodies[b].hull);
			for (uint32_t a : c.actions) {
				WkAct f = wk_action(a);
				if (!f) { fprintf(stderr, "action %u not valid for TL_WEAK\n", a); return 2; }
				bodies[b].add_action(f);
			}
		}
		run_loop(w, c, bodies);
	}
	return 0;
}

// ---------------------------------------------------------------- scenarios
void write_case(const char* path, const Case& c) {
	Writer w(path);
	w.raw("MFCASE1\0", 8);
	w.u32(c.method); w.u32(c.nbodies); w.u32(c.nsteps); w.u32(c.dump_every); w.u32(c.contact);
	w.u32((uint32_t)c.actions.size());
	for (uint32_t a : c.actions) w.u32(a);
	w.f64(c.dt);
	w.f64(c.nu); w.f64(c.E); w.f64(c.rho0);
	w.f64(c.wdeltap); w.f64(c.corr_exp); w.f64(c.mghn_eps);
	w.f64(c.alpha); w.f64(c.beta); w.f64(c.eta);
	w.f64(c.xsph_eps);
	w.u32(c.do_smooth);
	w.f64(c.nbh_h); w.f64(c.nbh_eps);
	w.f64(c.gp_h); w.f64(c.gp_rho);
	for (const BodyIn& b : c.bodies) {
		w.u32(b.n);
		for (int k = 0; k < NIN; k++) w.raw(b.a[k].data(), b.n * 8);
		w.u32((uint32_t)b.hull.size());
		w.raw(b.hull.data(), b.hull.size() * 4);
		w.u32((uint32_t)b.bcs.size());
		for (const BC& bc : b.bcs) {
			w.u32(bc.kind); w.f64(bc.v); w.u32((uint32_t)bc.idx.size());
			w.raw(bc.idx.data(), bc.idx.size() * 4);
		}
		w.u32(b.ex); w.u32(b.ey);
		if ((c.method == TL_WEAK && b.ex == 0) || (c.method == UL_WEAK && b.ex == 1)) {
			w.u32((uint32_t)(b.quads.size() / 4)); w.u32(b.order); w.u32(b.shape);
			w.raw(b.quads.data(), b.quads.size() * 4);
		}
		if (c.method == UL_WEAK || (c.method == TL_WEAK && b.ex == 0)) {
			w.u32(b.ngp);
			for (int k = 0; k < NIN; k++) w.raw(b.g[k].data(), b.ngp * 8);
		}
	}
}

template <typename T>
BodyIn capture(body<T>& b) {
	BodyIn in;
	in.n = b.get_num_part();
	T** p = b.get_particles();
	for (int k = 0; k < NIN; k++) in.a[k].resize(in.n);
	for (unsigned i = 0; i < in.n; i++) {
		double f[NIN] = {p[i]->x, p[i]->y, p[i]->X, p[i]->Y, p[i]->m, p[i]->rho, p[i]->h, p[i]->quad_weight,
		                 p[i]->vx, p[i]->vy, p[i]->Sxx, p[i]->Sxy, p[i]->Syy};
		for (int k = 0; k < NIN; k++) in.a[k][i] = f[k];
	}
	if (b.has_boundary()) {
		const unsigned* ix = b.get_boundary()->indexes();
		in.hull.assign(ix, ix + b.get_boundary()->num_bound());
	}
	return in;
}

void fill_consts(Case& c, simulation_data sd, double dt) {
	physical_constants pc = sd.get_physical_constants();
	correction_constants cc = sd.get_correction_constants();
	c.dt = dt;
	c.nu = pc.nu(); c.E = pc.E(); c.rho0 = pc.rho0();
	c.wdeltap = cc.get_monaghan_const().mghn_wdeltap();
	c.corr_exp = cc.get_monaghan_const().mghn_corr_exp();
	c.mghn_eps = cc.get_monaghan_const().mghn_eps();
	c.alpha = cc.get_art_visc_const().artvisc_alpha();
	c.beta = cc.get_art_visc_const().artvisc_beta();
	c.eta = cc.get_art_visc_const().artvisc_eta();
	c.xsph_eps = cc.xsph_eps();
	c.do_smooth = cc.do_smooth() ? 1 : 0;
}

int run_scenario(const std::string& name, unsigned nbox, unsigned nsteps, const char* case_out, const char* out) {
	Case c;
	c.nsteps = nsteps;
	c.nbh_eps = 1e-6;
	g_nbh.assign(2, {});
	g_recorded.assign(2, false);
	const std::vector<uint32_t> ul_actions = {RIEMANN_UPDATE_INTEGRATION_WEIGHTS, MATERIAL_EOS, CORRECTORS_MGHN_ARTIFICIAL_STRESS,
	                                          DERIVE_STRESS_MONAGHAN, DERIVE_VELOCITY, CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
	                                          CORRECTORS_XSPH, MATERIAL_STRESS_RATE_JAUMANN, CONTMECH_CONTINUITY,
	                                          CONTMECH_MOMENTUM_UL, CONTMECH_ADVECTION};  // rings.cpp:86-96,609-619
	if (name == "rings_monaghan" || name == "rings_monaghan_contact") {
		std::vector<body<particle_monaghan>> bodies = name == "rings_monaghan" ? rings_monaghan(nbox) : rings_monaghan_contact(nbox);
		c.method = UL;
		c.contact = name == "rings_monaghan_contact";
		c.actions = ul_actions;
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		for (auto& b : bodies) { c.bodies.push_back(capture(b)); b.add_action(&record_first_nbh<particle_monaghan>); }
		c.nbodies = (uint32_t)bodies.size();
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "rings_tl_contact") {
		std::vector<body<particle_tl>> bodies = rings_tl_contact(nbox);
		c.method = TL;
		c.contact = 1;
		c.actions = {DERIVE_DISPLACEMENT, MATERIAL_COMPUTE_STRESS_GREEN_STVENANT, CONTMECH_CAUCHY_TO_NOMINAL, DERIVE_STRESS_TL,
		             CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY, CONTMECH_MOMENTUM_TL, CONTMECH_ADVECTION};  // rings.cpp:419-425
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;  // hdx*dx, rings.cpp:404-407
		for (unsigned b = 0; b < bodies.size(); b++) {
			c.bodies.push_back(capture(bodies[b]));
			record_fixed_nbh(bodies[b].get_particles(), bodies[b].get_num_part(), (int)b);
		}
		c.nbodies = (uint32_t)bodies.size();
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "tensile_tl") {
		std::vector<body<particle_tl>> bodies = tensile_tl(nbox);
		c.method = TL;
		c.actions = {DERIVE_DISPLACEMENT, DERIVE_VELOCITY_TL, CONTMECH_VELOCITY_GRADIENT_TL, CONTMECH_CONTINUITY, MATERIAL_EOS,
		             MATERIAL_STRESS_RATE_JAUMANN, CONTMECH_CAUCHY_TO_NOMINAL, DERIVE_STRESS_TL,
		             CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY, CONTMECH_MOMENTUM_TL, CONTMECH_ADVECTION};  // tensile.cpp:276-286
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;
		BodyIn in = capture(bodies[0]);
		BC l, r;  // tensile.cpp:234-246,262-264
		l.kind = r.kind = BC_PULL_TL;
		l.v = -10.; r.v = 10.;
		for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
		in.bcs = {l, r};
		c.bodies.push_back(in);
		record_fixed_nbh(bodies[0].get_particles(), bodies[0].get_num_part(), 0);
		c.nbodies = 1;
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "rings_corot_contact" || name == "tensile_corot" || name == "rotation_corot") {
		const bool rings = name == "rings_corot_contact", disc = name == "rotation_corot";
		std::vector<body<particle_corotational>> bodies =
		    rings ? rings_corot_contact(nbox) : (disc ? rotation_corot(nbox) : tensile_corot(nbox));
		c.method = COROT;
		c.contact = rings ? 1 : 0;
		c.actions = {COROTATIONAL_ANISOTROPY_TENSOR, DERIVE_DISPLACEMENT_COROTATIONAL, MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN,
		             CONTMECH_CAUCHY_TO_NOMINAL, DERIVE_STRESS_COROTATIONAL, CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY,
		             CONTMECH_ADVECTION};  // rings.cpp:325-331, tensile.cpp:202-208
		if (disc)  // rotation.cpp:132-137: no artificial viscosity
			c.actions = {COROTATIONAL_ANISOTROPY_TENSOR, DERIVE_DISPLACEMENT_COROTATIONAL,
			             MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN, CONTMECH_CAUCHY_TO_NOMINAL, DERIVE_STRESS_COROTATIONAL,
			             CONTMECH_ADVECTION};
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;
		for (unsigned b = 0; b < bodies.size(); b++) {
			BodyIn in = capture(bodies[b]);
			if (!rings && !disc) {
				BC l, r;  // tensile.cpp:170-176,188-190
				l.kind = r.kind = BC_PULL_TL;
				l.v = -10.; r.v = 10.;
				for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
				in.bcs = {l, r};
			}
			c.bodies.push_back(in);
			record_fixed_nbh(bodies[b].get_particles(), bodies[b].get_num_part(), (int)b);
		}
		c.nbodies = (uint32_t)bodies.size();
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "rings_godunov" || name == "rings_godunov_contact" || name == "rotation_godunov") {
		std::vector<body<particle_ul>> bodies = name == "rings_godunov" ? rings_godunov(nbox)
		                                        : (name == "rotation_godunov" ? rotation_godunov(nbox)
		                                                                      : rings_godunov_contact(nbox));
		c.method = UL;
		c.contact = name == "rings_godunov_contact";
		c.actions = {RIEMANN_UPDATE_INTEGRATION_WEIGHTS, MATERIAL_EOS, DERIVE_VELOCITY, MATERIAL_STRESS_RATE_JAUMANN,
		             GODUNOV_CONTINUITY, GODUNOV_MOMENTUM, CONTMECH_ADVECTION};  // rings.cpp:154-160,233-239
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		for (auto& b : bodies) { c.bodies.push_back(capture(b)); b.add_action(&record_first_nbh<particle_ul>); }
		c.nbodies = (uint32_t)bodies.size();
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "tensile_godunov" || name == "tensile_monaghan" || name == "rotation_monaghan") {
		// UL plates pulled by the velocity conditions of tensile.cpp:44-66, and the
		// spinning UL disc; both run as particle_monaghan bodies here (the Godunov
		// actions take any particle_ul)
		std::vector<body<particle_monaghan>> bm;
		std::vector<body<particle_ul>> bu;
		c.method = UL;
		if (name == "tensile_godunov") {
			bu = tensile_godunov(nbox);
			c.actions = {RIEMANN_UPDATE_INTEGRATION_WEIGHTS, MATERIAL_EOS, DERIVE_VELOCITY, MATERIAL_STRESS_RATE_JAUMANN,
			             GODUNOV_CONTINUITY, GODUNOV_MOMENTUM, CONTMECH_ADVECTION};  // tensile.cpp:126-132
			fill_consts(c, bu[0].get_sim_data(), simulation_time::getInstance().get_dt());
			c.bodies.push_back(capture(bu[0]));
			bu[0].add_action(&record_first_nbh<particle_ul>);
		} else {
			bm = name == "tensile_monaghan" ? tensile_monaghan(nbox) : rotation_monaghan(nbox);
			c.actions = ul_actions;  // tensile.cpp:437-447, rotation.cpp:338-348
			fill_consts(c, bm[0].get_sim_data(), simulation_time::getInstance().get_dt());
			c.bodies.push_back(capture(bm[0]));
			bm[0].add_action(&record_first_nbh<particle_monaghan>);
		}
		if (name != "rotation_monaghan") {
			// tensile.cpp:119-120 / :431-432; the Monaghan plate pulls three columns at
			// each end (tensile.cpp:392-398), the Godunov plate one (:97-103)
			const unsigned cols = name == "tensile_monaghan" ? 3 : 1;
			BC l, r;
			l.kind = r.kind = BC_VELOCITY_UL;
			l.v = -10.; r.v = 10.;
			for (unsigned i = 0; i < cols; i++)
				for (unsigned j = 0; j < nbox; j++) {
					l.idx.push_back(i * nbox + j);
					r.idx.push_back((nbox - cols + i) * nbox + j);
				}
			c.bodies[0].bcs = {l, r};
		}
		c.nbodies = 1;
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		if (bu.empty()) run_loop(w, c, bm);
		else run_loop(w, c, bu);
	} else if (name == "rotation_tl") {
		std::vector<body<particle_tl>> bodies = rotation_tl(nbox);
		c.method = TL;
		c.actions = {DERIVE_DISPLACEMENT, DERIVE_VELOCITY_TL, CONTMECH_VELOCITY_GRADIENT_TL, CONTMECH_CONTINUITY, MATERIAL_EOS,
		             MATERIAL_STRESS_RATE_JAUMANN, CONTMECH_CAUCHY_TO_NOMINAL, DERIVE_STRESS_TL,
		             CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY, CONTMECH_MOMENTUM_TL, CONTMECH_ADVECTION};  // rotation.cpp:196-206
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;
		c.bodies.push_back(capture(bodies[0]));
		record_fixed_nbh(bodies[0].get_particles(), bodies[0].get_num_part(), 0);
		c.nbodies = 1;
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "rings_potential_contact" || name == "tensile_potential" || name == "rotation_potential") {
		const bool rings = name == "rings_potential_contact", disc = name == "rotation_potential";
		std::vector<body<particle_potential>> bodies =
		    rings ? rings_potential_contact(nbox) : (disc ? rotation_potential(nbox) : tensile_potential(nbox));
		c.method = POTENTIAL;
		c.contact = rings ? 1 : 0;
		c.actions = {DERIVE_DISPLACEMENT, MATERIAL_COMPUTE_STRESS_GREEN_STVENANT, POTENTIAL_COMP_ELASTIC_POTENTIAL,
		             CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY, CONTMECH_ADVECTION};  // rings.cpp:512-516, tensile.cpp:354-358
		if (disc)  // rotation.cpp:266-269: no artificial viscosity
			c.actions = {DERIVE_DISPLACEMENT, MATERIAL_COMPUTE_STRESS_GREEN_STVENANT, POTENTIAL_COMP_ELASTIC_POTENTIAL,
			             CONTMECH_ADVECTION};
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;
		for (unsigned b = 0; b < bodies.size(); b++) {
			BodyIn in = capture(bodies[b]);
			if (!rings && !disc) {
				BC l, r;  // tensile.cpp:349-350
				l.kind = r.kind = BC_PULL_TL;
				l.v = -10.; r.v = 10.;
				for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
				in.bcs = {l, r};
			}
			c.bodies.push_back(in);
			record_fixed_nbh(bodies[b].get_particles(), bodies[b].get_num_part(), (int)b);
		}
		c.nbodies = (uint32_t)bodies.size();
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else if (name == "tensile_ul_weak" || name == "rotation_ul_weak" || name == "rings_ul_weak_contact") {
		typedef particle_ul_weak T;
		std::vector<body<T>> bodies = name == "tensile_ul_weak" ? tensile_ul_weak(nbox)
		                              : (name == "rotation_ul_weak" ? rotation_ul_weak(nbox) : rings_ul_weak_contact(nbox));
		c.method = UL_WEAK;
		c.contact = name == "rings_ul_weak_contact";
		// tensile.cpp:713-726; rotation.cpp:511-525 and rings.cpp:917-930 take the
		// momentum of cont_mech.h:51-68
		const uint32_t momentum = name == "tensile_ul_weak" ? CONTMECH_MOMENTUM_UL : CONTMECH_MOMENTUM_UL_WEAK;
		c.actions = {RIEMANN_UPDATE_INTEGRATION_WEIGHTS, RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP, MATERIAL_EOS_GP,
		             DERIVE_STRESS_WEAK_UL, DERIVE_VELOCITY_WEAK, DERIVE_VELOCITY, MATERIAL_STRESS_RATE_JAUMANN_GP,
		             momentum, CONTMECH_CONTINUITY, CONTMECH_CONTINUITY_GP, CONTMECH_ADVECTION,
		             INTERPOLATION_INTERPOLATE_VELOCITY, CONTMECH_ADVECTION_GP};
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = 1.5 * bodies[0].get_particles()[0]->h;  // find_neighbors(.., 1.5*dx, ..) with h = dx
		g_gp.assign(bodies.size(), BodyIn());
		g_gp_done.assign(bodies.size(), false);
		for (unsigned b = 0; b < bodies.size(); b++) {
			BodyIn in = capture(bodies[b]);
			if (name == "tensile_ul_weak") {
				BC l, r;  // tensile.cpp:688-690
				l.kind = r.kind = BC_VELOCITY_UL;
				l.v = -10.; r.v = 10.;
				for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
				in.bcs = {l, r};
			}
			c.bodies.push_back(in);
			std::vector<void (*)(body<T>&)> acts;
			bodies[b].add_action(&record_first_nbh<T>);
			bodies[b].add_action(&capture_gp<T>);
		}
		c.nbodies = (uint32_t)bodies.size();
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
		for (unsigned b = 0; b < bodies.size(); b++) {
			c.bodies[b].ngp = g_gp[b].n;
			for (int k = 0; k < NIN; k++) c.bodies[b].g[k] = g_gp[b].a[k];
		}
		write_case(case_out, c);
	} else if (name == "tensile_ul_fem" || name == "rotation_ul_fem" || name == "rings_ul_fem_contact") {
		// weak UL bodies with a gauss_int: bilinear elements on the rectangle
		// (tensile.cpp:452-537) or mesh_ring (rotation.cpp:353-405, rings.cpp:623-718),
		// 2x2 Gauss points placed again on the current nodes at every evaluation
		typedef particle_ul_weak T;
		const bool rings = name == "rings_ul_fem_contact", disc = name == "rotation_ul_fem";
		std::vector<body<T>> bodies = name == "tensile_ul_fem"   ? tensile_ul_fem(nbox)
		                              : disc ? rotation_ul_fem(nbox) : rings_ul_fem_contact(nbox);
		std::vector<element> elems;
		if (rings || disc) {
			unsigned nn = 0;
			T** tmp = mesh_ring<T>(nbox, nn, elems, rings ? 0.03 : 0., rings ? 0.04 : 1.);
			for (unsigned i = 0; i < nn; i++) delete tmp[i];
			delete[] tmp;
		} else {
			elems = element_map_rectangle(nbox - 1, nbox - 1);
		}
		c.method = UL_WEAK;
		c.contact = rings ? 1 : 0;
		c.actions = {MATERIAL_EOS_GP, DERIVE_STRESS_WEAK_UL, DERIVE_VELOCITY_WEAK, MATERIAL_STRESS_RATE_JAUMANN_GP,
		             CONTMECH_MOMENTUM_UL_WEAK, CONTMECH_CONTINUITY_GP, CONTMECH_ADVECTION};  // tensile.cpp:526-532
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = 0.;
		g_gp.assign(bodies.size(), BodyIn());
		g_gp_done.assign(bodies.size(), false);
		for (unsigned b = 0; b < bodies.size(); b++) {
			BodyIn in = capture(bodies[b]);
			in.ex = 1;
			in.ey = 0;
			in.order = 2;
			in.shape = SHAPE_ELEMENT;
			for (const element& e : elems) {
				in.quads.push_back(e.ll_idx); in.quads.push_back(e.lr_idx);
				in.quads.push_back(e.tr_idx); in.quads.push_back(e.tl_idx);
			}
			if (name == "tensile_ul_fem") {
				BC l, r;  // tensile.cpp:507-509
				l.kind = r.kind = BC_VELOCITY_UL;
				l.v = -10.; r.v = 10.;
				for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
				in.bcs = {l, r};
			}
			c.bodies.push_back(in);
			bodies[b].add_action(&record_first_nbh<T>);
			bodies[b].add_action(&capture_gp<T>);
		}
		c.nbodies = (uint32_t)bodies.size();
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
		for (unsigned b = 0; b < bodies.size(); b++) {
			c.bodies[b].ngp = g_gp[b].n;
			for (int k = 0; k < NIN; k++) c.bodies[b].g[k] = g_gp[b].a[k];
		}
		write_case(case_out, c);
	} else if (name == "tensile_tl_fem" || name == "rotation_tl_fem" || name == "rings_tl_fem_contact" ||
	           name == "rotation_tl_weak" || name == "rings_tl_weak_contact") {
		// weak TL bodies on explicit element maps: the rectangle (tensile.cpp:581) or
		// mesh_ring (rings.cpp:742-743, rotation.cpp:425,555), 2x2 Gauss points; the
		// *_fem set-ups keep the elements' shape functions, the *_weak ones use RKPM
		typedef particle_tl_weak T;
		const bool rings = name.compare(0, 6, "rings_") == 0, disc = name.compare(0, 9, "rotation_") == 0;
		const bool fem = name.find("_fem") != std::string::npos;
		std::vector<body<T>> bodies = name == "tensile_tl_fem"   ? tensile_tl_fem(nbox)
		                              : name == "rotation_tl_fem" ? rotation_tl_fem(nbox)
		                              : name == "rings_tl_fem_contact" ? rings_tl_fem_contact(nbox)
		                              : name == "rotation_tl_weak" ? rotation_tl_weak(nbox)
		                                                             : rings_tl_weak_contact(nbox);
		std::vector<element> elems;
		if (rings || disc) {
			unsigned nn = 0;
			T** tmp = mesh_ring<T>(nbox, nn, elems, rings ? 0.03 : 0., rings ? 0.04 : 1.);
			for (unsigned i = 0; i < nn; i++) delete tmp[i];
			delete[] tmp;
		} else {
			elems = element_map_rectangle(nbox - 1, nbox - 1);
		}
		c.method = TL_WEAK;
		c.contact = rings ? 1 : 0;
		c.actions = {DERIVE_DISPLACEMENT_WEAK, DERIVE_VELOCITY_TL_WEAK, CONTMECH_VELOCITY_GRADIENT_TL_GP, CONTMECH_CONTINUITY_GP,
		             MATERIAL_EOS_GP, MATERIAL_STRESS_RATE_JAUMANN_GP, CONTMECH_CAUCHY_TO_NOMINAL_GP, DERIVE_STRESS_WEAK_TL,
		             CONTMECH_MOMENTUM_TL_WEAK, CONTMECH_ADVECTION};  // rings.cpp:802-811 and the same lists
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = fem ? 0. : bodies[0].get_particles()[0]->h;  // find_neighbors(.., hdx*dx, ..)
		g_gp.assign(bodies.size(), BodyIn());
		g_gp_done.assign(bodies.size(), false);
		for (unsigned b = 0; b < bodies.size(); b++) {
			BodyIn in = capture(bodies[b]);
			in.ex = in.ey = 0;
			in.order = 2;
			in.shape = fem ? SHAPE_ELEMENT : SHAPE_RKPM;
			for (const element& e : elems) {
				in.quads.push_back(e.ll_idx); in.quads.push_back(e.lr_idx);
				in.quads.push_back(e.tr_idx); in.quads.push_back(e.tl_idx);
			}
			if (name == "tensile_tl_fem") {
				BC l, r;  // tensile.cpp:595-596
				l.kind = r.kind = BC_PULL_TL;
				l.v = -10.; r.v = 10.;
				for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
				in.bcs = {l, r};
			}
			c.bodies.push_back(in);
			record_fixed_nbh(bodies[b].get_particles(), bodies[b].get_num_part(), (int)b);
			bodies[b].add_action(&capture_gp_tl<T>);
		}
		c.nbodies = (uint32_t)bodies.size();
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
		for (unsigned b = 0; b < bodies.size(); b++) {
			c.bodies[b].ngp = g_gp[b].n;
			for (int k = 0; k < NIN; k++) c.bodies[b].g[k] = g_gp[b].a[k];
		}
		write_case(case_out, c);
	} else if (name == "tensile_tl_weak") {
		std::vector<body<particle_tl_weak>> bodies = tensile_tl_weak(nbox);
		c.method = TL_WEAK;
		c.actions = {DERIVE_DISPLACEMENT_WEAK, DERIVE_VELOCITY_TL_WEAK, CONTMECH_VELOCITY_GRADIENT_TL_GP, CONTMECH_CONTINUITY_GP,
		             MATERIAL_EOS_GP, MATERIAL_STRESS_RATE_JAUMANN_GP, CONTMECH_CAUCHY_TO_NOMINAL_GP, DERIVE_STRESS_WEAK_TL,
		             CONTMECH_MOMENTUM_TL_WEAK, CONTMECH_ADVECTION};  // tensile.cpp:814-823
		fill_consts(c, bodies[0].get_sim_data(), simulation_time::getInstance().get_dt());
		c.nbh_h = bodies[0].get_particles()[0]->h;
		c.gp_h = bodies[0].get_particles()[0]->h;  // Gauss points get hdx*dx too, tensile.cpp:792-795
		c.gp_rho = c.rho0;
		BodyIn in = capture(bodies[0]);
		in.ex = nbox - 1; in.ey = nbox - 1;
		BC l, r;
		l.kind = r.kind = BC_PULL_TL;
		l.v = -10.; r.v = 10.;
		for (unsigned i = 0; i < nbox; i++) { l.idx.push_back(i); r.idx.push_back((nbox - 1) * nbox + i); }
		in.bcs = {l, r};
		c.bodies.push_back(in);
		record_fixed_nbh(bodies[0].get_particles(), bodies[0].get_num_part(), 0);
		c.nbodies = 1;
		write_case(case_out, c);
		Writer w(out);
		write_header(w, c);
		run_loop(w, c, bodies);
	} else {
		fprintf(stderr, "unknown scenario %s\n", name.c_str());
		return 2;
	}
	return 0;
}

}  // namespace

int main(int argc, char** argv) {
	if (argc >= 4 && std::string(argv[1]) == "run") {
		Case c = read_case(argv[2]);
		if (argc >= 5) g_vtk_dir = argv[4];
		return run_case(c, argv[3]);
	}
	if (argc >= 7 && std::string(argv[1]) == "scenario")
		return run_scenario(argv[2], (unsigned)atoi(argv[3]), (unsigned)atoi(argv[4]), argv[5], argv[6]);
	fprintf(stderr, "usage: %s run CASE RESULT [VTKDIR] | scenario NAME NBOX NSTEPS CASE_OUT RESULT\n", argv[0]);
	return 2;
}
