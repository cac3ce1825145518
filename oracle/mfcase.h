// Test infrastructure: the binary "case" and "result" files shared by the CPU
// oracle (oracle/mfo.cpp), the harness that drives the compiled reference
// (oracle/ref_harness.cpp) and the Python tests.  Nothing in the product reads
// these files.
//
// A case describes one run of mfree_iwf's explicit time-step loop: the method,
// the simulation constants (simulation_data.h:25-99), the ordered action list
// (body::add_action, body.h:219-221), the initial particle state of every body,
// the contact boundary (convex-hull indices) and Dirichlet boundary conditions.
// All integers are little-endian uint32, all reals IEEE-754 binary64.
#ifndef MF_CASE_H
#define MF_CASE_H

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace mfcase {

enum Method : uint32_t { UL = 1, TL = 2, TL_WEAK = 3, COROT = 4, POTENTIAL = 5, UL_WEAK = 6 };

// Action identifiers; the numbering is the C ABI's mf_action (include/mfree_gb300.h).
enum Action : uint32_t {
	RIEMANN_UPDATE_INTEGRATION_WEIGHTS = 1,
	MATERIAL_EOS = 2,
	CORRECTORS_MGHN_ARTIFICIAL_STRESS = 3,
	DERIVE_STRESS_MONAGHAN = 4,
	DERIVE_VELOCITY = 5,
	CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY = 6,
	CORRECTORS_XSPH = 7,
	MATERIAL_STRESS_RATE_JAUMANN = 8,
	CONTMECH_CONTINUITY = 9,
	CONTMECH_MOMENTUM_UL = 10,
	CONTMECH_ADVECTION = 11,
	DERIVE_DISPLACEMENT = 12,
	MATERIAL_COMPUTE_STRESS_GREEN_STVENANT = 13,
	CONTMECH_CAUCHY_TO_NOMINAL = 14,
	DERIVE_STRESS_TL = 15,
	CONTMECH_MOMENTUM_TL = 16,
	DERIVE_VELOCITY_TL = 17,
	CONTMECH_VELOCITY_GRADIENT_TL = 18,
	DERIVE_DISPLACEMENT_WEAK = 19,
	DERIVE_VELOCITY_TL_WEAK = 20,
	CONTMECH_VELOCITY_GRADIENT_TL_GP = 21,
	CONTMECH_CONTINUITY_GP = 22,
	MATERIAL_EOS_GP = 23,
	MATERIAL_STRESS_RATE_JAUMANN_GP = 24,
	CONTMECH_CAUCHY_TO_NOMINAL_GP = 25,
	DERIVE_STRESS_WEAK_TL = 26,
	CONTMECH_MOMENTUM_TL_WEAK = 27,
	COROTATIONAL_ANISOTROPY_TENSOR = 28,
	DERIVE_DISPLACEMENT_COROTATIONAL = 29,
	MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN = 30,
	DERIVE_STRESS_COROTATIONAL = 31,
	GODUNOV_CONTINUITY = 32,
	GODUNOV_MOMENTUM = 33,
	POTENTIAL_COMP_ELASTIC_POTENTIAL = 34,
	RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP = 35,
	DERIVE_STRESS_WEAK_UL = 36,
	DERIVE_VELOCITY_WEAK = 37,
	CONTMECH_MOMENTUM_UL_WEAK = 38,
	INTERPOLATION_INTERPOLATE_VELOCITY = 39,
	CONTMECH_ADVECTION_GP = 40,
	ACTION_MAX = 41
};

// Boundary-condition kinds.  PULL_TL is the position-prescribed pull of
// tensile.cpp:20-42: x = X + v*t, y = Y, vx = v, vy = 0, vx_t = vy_t = 0.
// VELOCITY_UL is the updated-Lagrangian form of tensile.cpp:44-66: x_t = v, y_t = 0,
// vx = v, vy = 0, vx_t = vy_t = 0.
enum BCKind : uint32_t { BC_PULL_TL = 1, BC_VELOCITY_UL = 2 };

enum Shape : uint32_t { SHAPE_RKPM = 0, SHAPE_ELEMENT = 1 };

struct BC {
	uint32_t kind = 0;
	double v = 0.;
	std::vector<uint32_t> idx;
};

// the 13 per-particle input arrays, in file order
static const int NIN = 13;
static const char* const IN_NAMES[NIN] = {"x", "y", "X", "Y", "m", "rho", "h", "quad_weight", "vx", "vy", "Sxx", "Sxy", "Syy"};
// the 10 per-particle output arrays of every dump, in file order
static const int NOUT = 10;
static const char* const OUT_NAMES[NOUT] = {"x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy", "fcx", "fcy"};

struct BodyIn {
	uint32_t n = 0;
	std::vector<double> a[NIN];
	std::vector<uint32_t> hull;
	std::vector<BC> bcs;
	uint32_t ex = 0, ey = 0;  // TL_WEAK: element_map_rectangle(ex, ey), 2x2 Gauss points
	// TL_WEAK with ex = ey = 0: an explicit element map (ll, lr, tr, tl per element), the
	// Gauss order per direction, and the shape functions of the Gauss points
	// (SHAPE_RKPM: neighbour search + RKPM as tensile_tl_weak; SHAPE_ELEMENT: the
	// elements' own bilinear functions, as the *_fem set-ups)
	std::vector<uint32_t> quads;
	uint32_t order = 2, shape = 0;
	// UL_WEAK: the stress points; TL_WEAK with an explicit map: the Gauss points as the
	// set-up left them (x, y, X, Y, h, rho are read) -- their NIN arrays
	uint32_t ngp = 0;
	std::vector<double> g[NIN];
};

struct Case {
	uint32_t method = UL, nbodies = 0, nsteps = 0, dump_every = 0, contact = 0;
	std::vector<uint32_t> actions;
	double dt = 0.;
	double nu = 0., E = 0., rho0 = 0.;
	double wdeltap = 0., corr_exp = 0., mghn_eps = 0.;
	double alpha = 0., beta = 0., eta = 0.;
	double xsph_eps = 0.;
	uint32_t do_smooth = 0;
	double nbh_h = 0.;     // TL/TL_WEAK: the h given to find_neighbors (neighbor_search.h:116)
	double nbh_eps = 1e-6; // absolute epsilon of the neighbour predicate (grid.h:157, neighbor_search.h:41)
	double gp_h = 0., gp_rho = 0.;  // TL_WEAK: h and rho given to the Gauss points (tensile.cpp:792-795)
	                                // (UL_WEAK: nbh_h is the h of the Manhattan candidate search)
	std::vector<BodyIn> bodies;
};

struct Reader {
	FILE* f;
	explicit Reader(const char* path) : f(fopen(path, "rb")) {
		if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
	}
	~Reader() { if (f) fclose(f); }
	void raw(void* p, size_t n) {
		if (n && fread(p, 1, n, f) != n) { fprintf(stderr, "truncated case file\n"); exit(2); }
	}
	uint32_t u32() { uint32_t v; raw(&v, 4); return v; }
	double f64() { double v; raw(&v, 8); return v; }
	void vu32(std::vector<uint32_t>& v, size_t n) { v.resize(n); raw(v.data(), n * 4); }
	void vf64(std::vector<double>& v, size_t n) { v.resize(n); raw(v.data(), n * 8); }
};

inline Case read_case(const char* path) {
	Reader r(path);
	char magic[8];
	r.raw(magic, 8);
	if (memcmp(magic, "MFCASE1", 7) != 0) { fprintf(stderr, "bad case magic\n"); exit(2); }
	Case c;
	c.method = r.u32(); c.nbodies = r.u32(); c.nsteps = r.u32(); c.dump_every = r.u32(); c.contact = r.u32();
	uint32_t na = r.u32();
	r.vu32(c.actions, na);
	c.dt = r.f64();
	c.nu = r.f64(); c.E = r.f64(); c.rho0 = r.f64();
	c.wdeltap = r.f64(); c.corr_exp = r.f64(); c.mghn_eps = r.f64();
	c.alpha = r.f64(); c.beta = r.f64(); c.eta = r.f64();
	c.xsph_eps = r.f64();
	c.do_smooth = r.u32();
	c.nbh_h = r.f64(); c.nbh_eps = r.f64();
	c.gp_h = r.f64(); c.gp_rho = r.f64();
	c.bodies.resize(c.nbodies);
	for (auto& b : c.bodies) {
		b.n = r.u32();
		for (int k = 0; k < NIN; k++) r.vf64(b.a[k], b.n);
		uint32_t nh = r.u32();
		r.vu32(b.hull, nh);
		uint32_t nbc = r.u32();
		b.bcs.resize(nbc);
		for (auto& bc : b.bcs) {
			bc.kind = r.u32();
			bc.v = r.f64();
			uint32_t k = r.u32();
			r.vu32(bc.idx, k);
		}
		b.ex = r.u32(); b.ey = r.u32();
		// an explicit element map: TL_WEAK bodies without a rectangle, UL_WEAK bodies
		// with ex = 1 (a gauss_int in place of the ellipse, the *_ul_fem set-ups)
		if ((c.method == TL_WEAK && b.ex == 0) || (c.method == UL_WEAK && b.ex == 1)) {
			uint32_t ne = r.u32();
			b.order = r.u32();
			b.shape = r.u32();
			r.vu32(b.quads, 4 * (size_t)ne);
		}
		if (c.method == UL_WEAK || (c.method == TL_WEAK && b.ex == 0)) {
			b.ngp = r.u32();
			for (int k = 0; k < NIN; k++) r.vf64(b.g[k], b.ngp);
		}
	}
	return c;
}

// Result file: "MFOUT1\0\0", nbodies, ndumps, then per dump (step, time, per body
// the NOUT arrays), then per body the neighbour lists of the first derivative
// evaluation (UL) or of the set-up (TL): n, counts[n], concatenated idx lists.
struct Writer {
	FILE* f;
	explicit Writer(const char* path) : f(fopen(path, "wb")) {
		if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
	}
	~Writer() { if (f) fclose(f); }
	void raw(const void* p, size_t n) { if (n) fwrite(p, 1, n, f); }
	void u32(uint32_t v) { raw(&v, 4); }
	void f64(double v) { raw(&v, 8); }
};

}  // namespace mfcase

#endif
