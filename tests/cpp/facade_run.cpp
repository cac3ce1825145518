// Test program: runs a case file (the oracle's format, oracle/mfcase.h) through the
// header-only C++ facade include/mfree_gb300.hpp, written the way the reference's
// scenario code is (body + add_action + set_boundary), and writes the final state as
// a result file the tests compare with the oracle's.
//
//   facade_run CASE RESULT [fp64_strict|fp64|mixed]
#include <cstdio>
#include <cstring>

#include "../../include/mfree_gb300.hpp"
#include "../../oracle/mfcase.h"

int main(int argc, char** argv) {
	if (argc < 3) {
		fprintf(stderr, "usage: facade_run CASE RESULT [precision]\n");
		return 2;
	}
	mf_precision prec = MF_PREC_FP64_STRICT;
	if (argc > 3 && !strcmp(argv[3], "fp64")) prec = MF_PREC_FP64;
	if (argc > 3 && !strcmp(argv[3], "mixed")) prec = MF_PREC_MIXED;
	mfcase::Case cs = mfcase::read_case(argv[1]);
	try {
		mf::context ctx((mf_method)cs.method, prec, 0, cs.contact != 0, cs.nbh_eps, cs.nbh_h);
		mf_sim_data sd = {cs.nu, cs.E, cs.rho0, cs.wdeltap, cs.corr_exp, cs.mghn_eps, cs.alpha,
		                  cs.beta, cs.eta, cs.xsph_eps, (int32_t)cs.do_smooth, 0};
		std::vector<mf::body> bodies;
		for (auto& b : cs.bodies) {
			auto& a = b.a;  // x y X Y m rho h quad_weight vx vy Sxx Sxy Syy
			mf_particles p = {a[0].data(), a[1].data(), a[2].data(), a[3].data(), a[4].data(),
			                  a[5].data(), a[6].data(), a[7].data(), a[8].data(), a[9].data(),
			                  a[10].data(), a[11].data(), a[12].data()};
			mf::body body = ctx.add_body(p, b.n, sd, cs.dt);
			if (!b.hull.empty()) body.set_boundary(b.hull);
			for (auto& bc : b.bcs) body.add_boundary_condition(bc.idx, (mf_bc_kind)bc.kind, bc.v);
			for (uint32_t act : cs.actions) body.add_action((mf::action)act);
			if (cs.method == mfcase::TL_WEAK && b.ex) body.set_gauss_mesh(b.ex, b.ey, cs.gp_h, cs.gp_rho);
			if (cs.method == mfcase::TL_WEAK && !b.ex) {
				body.set_elements(b.quads, b.order, (int32_t)b.shape, cs.gp_h, cs.gp_rho);
				if (b.ngp) body.set_gauss_points(b.g[0], b.g[1], b.g[6], b.g[5]);
			}
			if (cs.method == mfcase::UL_WEAK) {
				if (b.ex == 1) body.set_elements(b.quads, b.order, MF_SHAPE_ELEMENT);
				auto& g = b.g;
				mf_particles sp = {g[0].data(), g[1].data(), g[2].data(), g[3].data(), g[4].data(),
				                   g[5].data(), g[6].data(), g[7].data(), g[8].data(), g[9].data(),
				                   g[10].data(), g[11].data(), g[12].data()};
				body.set_stress_points(sp, b.ngp);
			}
			bodies.push_back(body);
		}
		ctx.step((int32_t)cs.nsteps);
		mfcase::Writer w(argv[2]);
		w.raw("MFOUT1\0\0", 8);
		w.u32((uint32_t)bodies.size());
		for (auto& b : bodies) w.u32(b.get_num_part());
		w.u32(1);
		w.u32(cs.nsteps);
		w.f64(bodies.empty() ? 0. : bodies[0].get_time());
		for (auto& b : bodies) {
			mf::state s = b.get_state();
			const std::vector<double>* f[10] = {&s.x, &s.y, &s.vx, &s.vy, &s.rho, &s.Sxx, &s.Sxy, &s.Syy, &s.fcx, &s.fcy};
			for (auto* v : f) w.raw(v->data(), v->size() * 8);
		}
		w.u32(0);
	} catch (const mf::error& e) {
		fprintf(stderr, "%s\n", e.what());
		return e.status == MF_ERR_NO_DEVICE ? 3 : 1;
	}
	return 0;
}
