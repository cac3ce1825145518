// ORACLE -- test infrastructure only.  A CPU restatement, in structure-of-arrays
// form, of mfree_iwf's explicit meshless time step.  Only the tests, the smoke
// check and the CPU-baseline leg of the benchmark run it, as the checker; the
// product never links, calls or ships it.
//
// It restates, function by function, the reference code named beside each
// routine (paths relative to the reference's src/).  A particle "object" of the
// reference is a slot of a PSet; the reference's arrays of particle pointers are
// modelled by a permutation `perm` (array position -> slot), so that sorting the
// pointer array (body.h:137,147) sorts `perm` with the same comparator and the
// same std::sort -- the within-cell order, hence every floating-point summation
// order, is then the reference's own.  The vector/matrix arithmetic that the
// reference takes from GLM comes from the project-written subset in
// oracle/glm_subset, the same header the compiled reference uses.  Built with
// -ffp-contract=off so that x86-64 and aarch64 hosts round identically.
//
// Usage: mfo_run CASE_FILE RESULT_FILE [WARMUP_STEPS]
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <glm/glm.hpp>

#include "mfcase.h"

using namespace mfcase;

namespace {

const unsigned MAX_NBH = 200;  // particle.h:31

// ------------------------------------------------------------------ particles
// Fields of particle/particle_tl/particle_ul/particle_monaghan (particle.h:33-149).
struct PSet {
	unsigned n = 0;
	std::vector<unsigned> idx, hash;
	std::vector<double> x, y, X, Y, m, rho, h, qw, p, vx, vy, Sxx, Sxy, Syy;
	std::vector<double> vx_x, vx_y, vy_x, vy_y;
	std::vector<double> x_t, y_t, rho_t, vx_t, vy_t, Sxx_t, Sxy_t, Syy_t;
	std::vector<double> fcx, fcy;
	std::vector<double> Sxx_x, Sxy_y, Sxy_x, Syy_y;  // particle_ul
	std::vector<double> Rxx, Rxy, Ryy;               // particle_monaghan (particle_corotational: rotation R)
	std::vector<double> Ryx;                         // particle_corotational
	std::vector<double> Hxx, Hxy, Hyx, Hyy, Fdxx, Fdxy, Fdyx, Fdyy;  // particle_tl
	std::vector<double> Pxx, Pxy, Pyx, Pyy, Pxx_x, Pxy_x, Pyx_y, Pyy_y;
	std::vector<unsigned> num_nbh, nbh;  // nbh[slot*MAX_NBH + k]
	std::vector<double> w, w_x, w_y;
	std::vector<double> wji_x, wji_y;  // particle_potential: grad W of the reverse pair (particle.h:101)
	std::vector<unsigned> num_cand, cand;  // particle_ul_weak: candidate neighbours (particle.h:135-136)

	void resize(unsigned nn) {
		n = nn;
		for (auto* v : {&idx, &hash, &num_nbh, &num_cand}) v->assign(n, 0u);
		cand.assign((size_t)n * MAX_NBH, 0u);
		for (auto* v : {&x, &y, &X, &Y, &m, &rho, &h, &qw, &p, &vx, &vy, &Sxx, &Sxy, &Syy, &vx_x, &vx_y, &vy_x, &vy_y,
		                &x_t, &y_t, &rho_t, &vx_t, &vy_t, &Sxx_t, &Sxy_t, &Syy_t, &fcx, &fcy, &Sxx_x, &Sxy_y, &Sxy_x,
		                &Syy_y, &Rxx, &Rxy, &Ryy, &Ryx, &Hxx, &Hxy, &Hyx, &Hyy, &Fdxx, &Fdxy, &Fdyx, &Fdyy, &Pxx, &Pxy, &Pyx,
		                &Pyy, &Pxx_x, &Pxy_x, &Pyx_y, &Pyy_y})
			v->assign(n, 0.);
		nbh.assign((size_t)n * MAX_NBH, 0u);
		w.assign((size_t)n * MAX_NBH, 0.);
		w_x.assign((size_t)n * MAX_NBH, 0.);
		w_y.assign((size_t)n * MAX_NBH, 0.);
		wji_x.assign((size_t)n * MAX_NBH, 0.);
		wji_y.assign((size_t)n * MAX_NBH, 0.);
		for (unsigned i = 0; i < n; i++) idx[i] = i;
	}

	// particle::reset, particle.cpp:34-43
	void reset(unsigned s) {
		x_t[s] = 0.; y_t[s] = 0.; rho_t[s] = 0.; vx_t[s] = 0.; vy_t[s] = 0.;
		Sxx_t[s] = 0.; Sxy_t[s] = 0.; Syy_t[s] = 0.;
	}
};

// particle::copy_into (particle.cpp:45-74) plus the particle_tl (:106-116),
// particle_potential (:156-163), particle_ul_weak (:195-203) and particle_monaghan
// (:219-228) overrides: the union of the fields they copy.
void copy_into(const PSet& a, unsigned s, PSet& b, unsigned d) {
	b.idx[d] = a.idx[s]; b.hash[d] = a.hash[s];
	b.m[d] = a.m[s]; b.rho[d] = a.rho[s]; b.h[d] = a.h[s]; b.qw[d] = a.qw[s]; b.p[d] = a.p[s];
	b.x[d] = a.x[s]; b.y[d] = a.y[s]; b.X[d] = a.X[s]; b.Y[d] = a.Y[s];
	b.vx[d] = a.vx[s]; b.vy[d] = a.vy[s];
	b.Sxx[d] = a.Sxx[s]; b.Sxy[d] = a.Sxy[s]; b.Syy[d] = a.Syy[s];
	b.fcx[d] = a.fcx[s]; b.fcy[d] = a.fcy[s];
	unsigned nn = a.num_nbh[s];
	b.num_nbh[d] = nn;
	size_t so = (size_t)s * MAX_NBH, dof = (size_t)d * MAX_NBH;
	for (unsigned k = 0; k < nn; k++) {
		b.nbh[dof + k] = a.nbh[so + k];
		b.w[dof + k] = a.w[so + k]; b.w_x[dof + k] = a.w_x[so + k]; b.w_y[dof + k] = a.w_y[so + k];
		b.wji_x[dof + k] = a.wji_x[so + k]; b.wji_y[dof + k] = a.wji_y[so + k];
	}
	b.Pxx[d] = a.Pxx[s]; b.Pxy[d] = a.Pxy[s]; b.Pyx[d] = a.Pyx[s]; b.Pyy[d] = a.Pyy[s];
	b.Rxx[d] = a.Rxx[s]; b.Rxy[d] = a.Rxy[s]; b.Ryy[d] = a.Ryy[s]; b.Ryx[d] = a.Ryx[s];
	unsigned nc = a.num_cand[s];
	b.num_cand[d] = nc;
	for (unsigned k = 0; k < nc; k++) b.cand[dof + k] = a.cand[so + k];
}

struct Fail {
	const char* what;
};

// --------------------------------------------------------------------- kernel
// cubic_spline, kernel.cpp:20-55
struct KR {
	double w, w_x, w_y;
};
KR cubic_spline(double xi, double yi, double xj, double yj, double h) {
	double h1 = 1. / h;
	double xij = xi - xj;
	double yij = yi - yj;
	double rij = sqrt(xij * xij + yij * yij);
	double fac = 10 * (M_1_PI) / 7.0 * h1 * h1;
	double q = rij * h1;
	KR w{0., 0., 0.};
	if (q >= 2.) {
		return w;
	} else if (q >= 1.) {
		w.w = fac * (0.25 * (2 - q) * (2 - q) * (2 - q));
		if (rij > 1e-12) {
			double der = -0.75 * (2 - q) * (2 - q) * h1 / rij;
			w.w_x = xij * der * fac;
			w.w_y = yij * der * fac;
		}
		return w;
	} else {
		w.w = fac * (1 - 1.5 * q * q * (1 - 0.5 * q));
		if (rij > 1e-12) {
			double der = -3.0 * q * (1 - 0.75 * q) * h1 / rij;
			w.w_x = xij * der * fac;
			w.w_y = yij * der * fac;
		}
		return w;
	}
}

// ------------------------------------------------------------------ constants
// physical_constants, simulation_data.cpp:32-47
struct Consts {
	double nu, E, rho0;
	double G() const { return E / (2. * (1. + nu)); }
	double K() const { double g = G(); return 2.0 * g * (1 + nu) / (3 * (1 - 2 * nu)); }
	double c0() const { return sqrt(K() / rho0); }
};

// ----------------------------------------------------------------------- grid
// grid<T>, grid.h:28-191
struct Grid {
	double dx, lx, ly;
	unsigned nx, ny, num_cell;
	double bbmin_x, bbmax_x, bbmin_y, bbmax_y;

	// grid.h:83-115
	void update_geometry(const PSet& P, const std::vector<unsigned>& perm, double kernel_width) {
		bbmin_x = DBL_MAX; bbmax_x = -DBL_MAX;
		bbmin_y = DBL_MAX; bbmax_y = -DBL_MAX;
		double h_max = -DBL_MAX;
		for (unsigned i = 0; i < P.n; i++) {
			unsigned s = perm[i];
			bbmin_x = fmin(P.x[s], bbmin_x);
			bbmin_y = fmin(P.y[s], bbmin_y);
			bbmax_x = fmax(P.x[s], bbmax_x);
			bbmax_y = fmax(P.y[s], bbmax_y);
			h_max = fmax(P.h[s], h_max);
		}
		bbmin_x -= 1e-6; bbmin_y -= 1e-6;
		bbmax_x += 1e-6; bbmax_y += 1e-6;
		dx = h_max * kernel_width;
		lx = bbmax_x - bbmin_x;
		ly = bbmax_y - bbmin_y;
		nx = ceil(lx / dx);
		ny = ceil(ly / dx);
		num_cell = nx * ny;
		if (!(num_cell < P.n)) throw Fail{"grid: num_cell >= n (grid.h:114)"};
	}
	// grid.h:35-41
	void assign_hashes(PSet& P, const std::vector<unsigned>& perm) const {
		for (unsigned i = 0; i < P.n; i++) {
			unsigned s = perm[i];
			unsigned ix = (unsigned)((P.x[s] - bbmin_x) / dx);
			unsigned iy = (unsigned)((P.y[s] - bbmin_y) / dx);
			P.hash[s] = ix * ny + iy;
		}
	}
	// grid.h:48-81
	std::vector<int> get_cells(const PSet& P, const std::vector<unsigned>& perm) const {
		unsigned n = P.n;
		for (unsigned i = 0; i + 1 < n; i++)
			if (!(P.hash[perm[i]] <= P.hash[perm[i + 1]])) throw Fail{"grid: unsorted hashes (grid.h:52)"};
		std::vector<int> cells(num_cell + 1, -1);
		cells[P.hash[perm[0]]] = 0;
		for (unsigned i = 0; i + 1 < n; i++)
			if (P.hash[perm[i]] != P.hash[perm[i + 1]]) cells[P.hash[perm[i + 1]]] = i + 1;
		cells[P.hash[perm[n - 1]] + 1] = n;
		unsigned fix = n;
		for (auto it = cells.rbegin(); it != cells.rend(); ++it) {
			if (*it == -1) *it = fix;
			else fix = *it;
		}
		return cells;
	}
	// grid.h:117-177; eps is the absolute term of the predicate (1e-6 in the reference)
	void construct_verlet_lists(PSet& P, const std::vector<unsigned>& perm, double eps) const {
		std::vector<int> cells = get_cells(P, perm);
		for (unsigned b = 0; b < num_cell; b++) {
			unsigned gi = b / ny;
			unsigned gj = b - gi * ny;
			int low_i = (int)gi - 1 < 0 ? 0 : (int)gi - 1;
			int low_j = (int)gj - 1 < 0 ? 0 : (int)gj - 1;
			int high_i = gi + 2 > nx ? nx : gi + 2;
			int high_j = gj + 2 > ny ? ny : gj + 2;
			for (int i = cells[b]; i < cells[b + 1]; i++) {
				unsigned si = perm[i];
				unsigned nbh_iter = 0;
				double hi = P.h[si], xi = P.x[si], yi = P.y[si];
				double radius2 = hi * hi * 2 * 2;
				for (int ni = low_i; ni < high_i; ni++)
					for (int nj = low_j; nj < high_j; nj++)
						for (int j = cells[ni * ny + nj]; j < cells[ni * ny + nj + 1]; j++) {
							unsigned sj = perm[j];
							double xij = xi - P.x[sj];
							double yij = yi - P.y[sj];
							double r2 = xij * xij + yij * yij;
							if (r2 <= radius2 + eps) {
								if (nbh_iter >= MAX_NBH) throw Fail{"grid: neighbour overflow (grid.h:167)"};
								P.nbh[(size_t)si * MAX_NBH + nbh_iter] = j;
								nbh_iter++;
							}
						}
				if (!(nbh_iter < MAX_NBH)) throw Fail{"grid: neighbour overflow (grid.h:167)"};
				if (!(nbh_iter > 0)) throw Fail{"grid: particle without neighbours (grid.h:168)"};
				P.num_nbh[si] = nbh_iter;
			}
		}
	}
};

// ----------------------------------------------------------- shape functions
// precomp_sph, precomp_shape_functions.h:210-229
void precomp_sph(PSet& P, const std::vector<unsigned>& perm) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double xi = P.x[si], yi = P.y[si], hi = P.h[si];
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			KR w = cubic_spline(xi, yi, P.x[sj], P.y[sj], hi);
			P.w[o] = w.w; P.w_x[o] = w.w_x; P.w_y[o] = w.w_y;
		}
	}
}

// precomp_randles_libersky, precomp_shape_functions.h:231-290 (array in idx order)
void precomp_randles_libersky(PSet& P) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned num_nbh = P.num_nbh[i];
		double xi = P.x[i], yi = P.y[i], hi = P.h[i];
		double C = 0.;
		for (unsigned j = 0; j < num_nbh; j++) {
			unsigned jdx = P.nbh[(size_t)i * MAX_NBH + j];
			double xj = P.x[jdx], yj = P.y[jdx];
			double volj = P.m[jdx] / P.rho[jdx];
			KR w = cubic_spline(xi, yi, xj, yj, hi);
			C += w.w * volj;
		}
		glm::dmat2x2 B(0);
		for (unsigned j = 0; j < num_nbh; j++) {
			unsigned jdx = P.nbh[(size_t)i * MAX_NBH + j];
			double xj = P.x[jdx], yj = P.y[jdx];
			double volj = P.m[jdx] / P.rho[jdx];
			KR w = cubic_spline(xi, yi, xj, yj, hi);
			B[0][0] += (xj - xi) * w.w_x * volj * 1. / C;
			B[1][0] += (xj - xi) * w.w_y * volj * 1. / C;
			B[0][1] += (yj - yi) * w.w_x * volj * 1. / C;
			B[1][1] += (yj - yi) * w.w_y * volj * 1. / C;
		}
		glm::dmat2x2 invB = glm::inverse(B);
		for (unsigned j = 0; j < num_nbh; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			KR w = cubic_spline(xi, yi, P.x[jdx], P.y[jdx], hi);
			P.w[o] = w.w * 1. / C;
			P.w_x[o] = (w.w_x * invB[0][0] + w.w_y * invB[1][0]) * 1. / C;
			P.w_y[o] = (w.w_x * invB[0][1] + w.w_y * invB[1][1]) * 1. / C;
		}
	}
}

// precomp_randles_libersky_symmetric, precomp_shape_functions.h:292-315: for every
// listed pair (i, j), the weight gradient that j's list holds for i (the first
// match; a pair missing from j's list keeps zero)
void precomp_randles_libersky_symmetric(PSet& P) {
	precomp_randles_libersky(P);
	for (unsigned i = 0; i < P.n; i++)
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			for (unsigned k = 0; k < P.num_nbh[jdx]; k++) {
				size_t q = (size_t)jdx * MAX_NBH + k;
				if (P.nbh[q] == i) {
					P.wji_x[o] = P.w_x[q];
					P.wji_y[o] = P.w_y[q];
					break;
				}
			}
		}
}

// solve3x3, precomp_shape_functions.h:31-50
void solve3x3(const glm::dmat3x3& M, const glm::dvec3& rhs, glm::dvec3& x) {
	double delta = M[0][0] * M[1][1] * M[2][2] + M[1][0] * M[2][1] * M[0][2] + M[2][0] * M[0][1] * M[1][2] -
	               M[0][2] * M[1][1] * M[2][0] - M[1][2] * M[2][1] * M[0][0] - M[2][2] * M[0][1] * M[1][0];
	double delta_x = rhs[0] * M[1][1] * M[2][2] + M[1][0] * M[2][1] * rhs[2] + M[2][0] * rhs[1] * M[1][2] -
	                 rhs[2] * M[1][1] * M[2][0] - M[1][2] * M[2][1] * rhs[0] - M[2][2] * rhs[1] * M[1][0];
	double delta_y = M[0][0] * rhs[1] * M[2][2] + rhs[0] * M[2][1] * M[0][2] + M[2][0] * M[0][1] * rhs[2] -
	                 M[0][2] * rhs[1] * M[2][0] - rhs[2] * M[2][1] * M[0][0] - M[2][2] * M[0][1] * rhs[0];
	double delta_z = M[0][0] * M[1][1] * rhs[2] + M[1][0] * rhs[1] * M[0][2] + rhs[0] * M[0][1] * M[1][2] -
	                 M[0][2] * M[1][1] * rhs[0] - M[1][2] * rhs[1] * M[0][0] - rhs[2] * M[0][1] * M[1][0];
	if (!(fabs(delta) > 0.)) throw Fail{"rkpm: singular moment matrix (precomp_shape_functions.h:45)"};
	x[0] = delta_x / delta;
	x[1] = delta_y / delta;
	x[2] = delta_z / delta;
}

// compute_rkpm_correctors, precomp_shape_functions.h:52-141; `from` holds the particles
void rkpm_correctors(const PSet& to, unsigned i, const PSet& from, glm::dvec3& C, glm::dvec3& C_x, glm::dvec3& C_y) {
	double xi = to.x[i], yi = to.y[i], hi = to.h[i];
	glm::dmat3x3 M(0.), M_x(0.), M_y(0.);
	for (unsigned j = 0; j < to.num_nbh[i]; j++) {
		unsigned jdx = to.nbh[(size_t)i * MAX_NBH + j];
		double mj = from.m[jdx], rhoj = from.rho[jdx];
		double xj = from.x[jdx], yj = from.y[jdx];
		double rx = xi - xj, ry = yi - yj;
		double rx_x = 1., rx_y = 0., ry_x = 0., ry_y = 1.;
		KR w = cubic_spline(xi, yi, xj, yj, hi);
		M[0][0] += w.w * mj / rhoj;
		M[0][1] += w.w * rx * mj / rhoj;
		M[0][2] += w.w * ry * mj / rhoj;
		M[1][0] += w.w * rx * mj / rhoj;
		M[2][0] += w.w * ry * mj / rhoj;
		M[1][1] += rx * rx * w.w * mj / rhoj;
		M[1][2] += rx * ry * w.w * mj / rhoj;
		M[2][1] += ry * rx * w.w * mj / rhoj;
		M[2][2] += ry * ry * w.w * mj / rhoj;

		M_x[0][0] += w.w_x * mj / rhoj;
		M_x[0][1] += w.w_x * rx * mj / rhoj + w.w * rx_x * mj / rhoj;
		M_x[0][2] += w.w_x * ry * mj / rhoj + w.w * rx_y * mj / rhoj;
		M_x[1][0] += w.w_x * rx * mj / rhoj + w.w * rx_x * mj / rhoj;
		M_x[2][0] += w.w_x * ry * mj / rhoj + w.w * rx_y * mj / rhoj;
		M_x[1][1] += rx * rx * w.w_x * mj / rhoj + w.w * (rx_x * rx + rx * rx_x) * mj / rhoj;
		M_x[1][2] += rx * ry * w.w_x * mj / rhoj + w.w * (rx_x * ry + rx * rx_y) * mj / rhoj;
		M_x[2][1] += rx * ry * w.w_x * mj / rhoj + w.w * (rx_y * rx + ry * rx_x) * mj / rhoj;
		M_x[2][2] += ry * ry * w.w_x * mj / rhoj + w.w * (rx_y * ry + ry * rx_y) * mj / rhoj;

		M_y[0][0] += w.w_y * mj / rhoj;
		M_y[0][1] += w.w_y * rx * mj / rhoj + w.w * ry_x * mj / rhoj;
		M_y[0][2] += w.w_y * ry * mj / rhoj + w.w * ry_y * mj / rhoj;
		M_y[1][0] += w.w_y * rx * mj / rhoj + w.w * ry_x * mj / rhoj;
		M_y[2][0] += w.w_y * ry * mj / rhoj + w.w * ry_y * mj / rhoj;
		M_y[1][1] += rx * rx * w.w_y * mj / rhoj + w.w * (ry_x * rx + rx * ry_x) * mj / rhoj;
		M_y[1][2] += rx * ry * w.w_y * mj / rhoj + w.w * (ry_x * ry + rx * ry_y) * mj / rhoj;
		M_y[2][1] += rx * ry * w.w_y * mj / rhoj + w.w * (ry_y * rx + ry * ry_x) * mj / rhoj;
		M_y[2][2] += ry * ry * w.w_y * mj / rhoj + w.w * (ry_y * ry + ry * ry_y) * mj / rhoj;
	}
	glm::dvec3 P(0.);
	P[0] = 1.;
	solve3x3(M, P, C);
	glm::dvec3 rhs_x = -M_x * C;
	glm::dvec3 rhs_y = -M_y * C;
	solve3x3(M, rhs_x, C_x);
	solve3x3(M, rhs_y, C_y);
}

// precomp_rkpm (both overloads), precomp_shape_functions.h:143-208
void precomp_rkpm(PSet& to, const PSet& from) {
	for (unsigned i = 0; i < to.n; i++) {
		glm::dvec3 C, C_x, C_y;
		rkpm_correctors(to, i, from, C, C_x, C_y);
		double xi = to.x[i], yi = to.y[i], hi = to.h[i];
		for (unsigned j = 0; j < to.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = to.nbh[o];
			double xj = from.x[jdx], yj = from.y[jdx];
			double rx = xi - xj, ry = yi - yj;
			double rx_x = 1., rx_y = 0., ry_x = 0., ry_y = 1.;
			KR w = cubic_spline(xi, yi, xj, yj, hi);
			double Corr = (rx * C[1] + ry * C[2]) + C[0];
			double Corr_x = (rx * C_x[1] + ry * C_x[2]) + rx_x * C[1] + rx_y * C[2] + C_x[0];
			double Corr_y = (rx * C_y[1] + ry * C_y[2]) + ry_x * C[1] + ry_y * C[2] + C_y[0];
			to.w[o] = Corr * w.w;
			to.w_x[o] = Corr_x * w.w + Corr * w.w_x;
			to.w_y[o] = Corr_y * w.w + Corr * w.w_y;
		}
	}
}

// find_neighbors (euclidean), neighbor_search.h:32-41,50-81,116-147.  The result
// is the brute-force one (ascending j); a cell grid only prunes candidates.
void find_neighbors(PSet& to, const PSet& from, double h, double eps) {
	double radius2 = h * h * 2 * 2;
	double reach = sqrt(radius2 + eps) * (1. + 1e-12) + 1e-300;
	double bminx = DBL_MAX, bminy = DBL_MAX, bmaxx = -DBL_MAX, bmaxy = -DBL_MAX;
	for (unsigned j = 0; j < from.n; j++) {
		bminx = fmin(bminx, from.x[j]); bminy = fmin(bminy, from.y[j]);
		bmaxx = fmax(bmaxx, from.x[j]); bmaxy = fmax(bmaxy, from.y[j]);
	}
	long gx = (long)((bmaxx - bminx) / reach) + 1, gy = (long)((bmaxy - bminy) / reach) + 1;
	std::vector<std::vector<unsigned>> cell((size_t)gx * gy);
	for (unsigned j = 0; j < from.n; j++) {
		long cx = (long)((from.x[j] - bminx) / reach), cy = (long)((from.y[j] - bminy) / reach);
		cell[(size_t)cx * gy + cy].push_back(j);
	}
	std::vector<unsigned> cand;
	for (unsigned i = 0; i < to.n; i++) {
		double xi = to.x[i], yi = to.y[i];
		long cx = (long)floor((xi - bminx) / reach), cy = (long)floor((yi - bminy) / reach);
		cand.clear();
		for (long a = cx - 1; a <= cx + 1; a++)
			for (long b = cy - 1; b <= cy + 1; b++) {
				if (a < 0 || b < 0 || a >= gx || b >= gy) continue;
				for (unsigned j : cell[(size_t)a * gy + b]) cand.push_back(j);
			}
		std::sort(cand.begin(), cand.end());
		unsigned nbh_iter = 0;
		for (unsigned j : cand) {
			double xij = xi - from.x[j];
			double yij = yi - from.y[j];
			double r2 = xij * xij + yij * yij;
			if (r2 <= radius2 + eps) {
				if (nbh_iter >= MAX_NBH) throw Fail{"find_neighbors: overflow (neighbor_search.h:142)"};
				to.nbh[(size_t)i * MAX_NBH + nbh_iter] = j;
				nbh_iter++;
			}
		}
		if (!(nbh_iter < MAX_NBH)) throw Fail{"find_neighbors: overflow (neighbor_search.h:142)"};
		if (!(nbh_iter > 0)) throw Fail{"find_neighbors: no neighbours (neighbor_search.h:143)"};
		to.num_nbh[i] = nbh_iter;
	}
}

// find_neighbors with distance_manhattan into the candidate lists of particle_ul_weak
// (neighbor_search.h:43-48, 84-113, 150-180): every "from" point with
// |dx| < 2h + 1e-6 and |dy| < 2h + 1e-6, ascending
void find_candidates(PSet& to, const PSet& from, double h) {
	for (unsigned i = 0; i < to.n; i++) {
		double xi = to.x[i], yi = to.y[i];
		unsigned nbh_iter = 0;
		for (unsigned j = 0; j < from.n; j++) {
			double xij = xi - from.x[j];
			double yij = yi - from.y[j];
			if (fabs(xij) < 2. * h + 1e-6 && fabs(yij) < 2. * h + 1e-6) {
				if (nbh_iter >= MAX_NBH) throw Fail{"find_neighbors: overflow (neighbor_search.h:176)"};
				to.cand[(size_t)i * MAX_NBH + nbh_iter] = j;
				nbh_iter++;
			}
		}
		if (!(nbh_iter < MAX_NBH)) throw Fail{"find_neighbors: overflow (neighbor_search.h:176)"};
		if (!(nbh_iter > 0)) throw Fail{"find_neighbors: no neighbours (neighbor_search.h:177)"};
		to.num_cand[i] = nbh_iter;
	}
}

// eigen, neighbor_ellipse.h:29-60: eigenvalues of the symmetric 2x2 A, ascending, and
// unit eigenvectors as the columns of V (only D[0][0], D[1][1] are set)
void eigen2(const glm::dmat2x2& A, glm::dmat2x2& V, glm::dmat2x2& D) {
	if (fabs(A[1][0]) < 1e-9 && fabs(A[0][1]) < 1e-9) {
		V = glm::dmat2x2(1.);
		D = glm::dmat2x2(A[0][0], 0., 0., A[1][1]);
		return;
	}
	double T = A[0][0] + A[1][1];
	double det = glm::determinant(A);
	double L1 = T / 2 + sqrt(T * T / 4 - det);
	double L2 = T / 2 - sqrt(T * T / 4 - det);
	double lambda1 = fmin(L1, L2);
	double lambda2 = fmax(L1, L2);
	D[0][0] = lambda1;
	D[1][1] = lambda2;
	if (fabs(A[1][0]) > 1e-12) {
		glm::dvec2 v1 = glm::normalize(glm::dvec2(lambda1 - A[1][1], A[0][1]));
		glm::dvec2 v2 = glm::normalize(glm::dvec2(lambda2 - A[1][1], A[0][1]));
		V = glm::dmat2x2(v1, v2);
	} else {
		glm::dvec2 v1 = glm::normalize(glm::dvec2(A[1][0], lambda1 - A[0][0]));
		glm::dvec2 v2 = glm::normalize(glm::dvec2(A[1][0], lambda2 - A[0][0]));
		V = glm::dmat2x2(v1, v2);
	}
}

// nbh_ellipse, neighbor_ellipse.h:62-127: h = half the largest candidate distance; the
// neighbours are the candidates inside the ellipse of semi-axes 1.6651 sqrt(lambda)
// along the eigenvectors of the candidates' mean offset product
void nbh_ellipse(PSet& to, const PSet& from) {
	for (unsigned i = 0; i < to.n; i++) {
		double px = to.x[i], py = to.y[i];
		double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
		double h = 0.;
		unsigned nc = to.num_cand[i];
		for (unsigned j = 0; j < nc; j++) {
			unsigned jdx = to.cand[(size_t)i * MAX_NBH + j];
			double dx = px - from.x[jdx], dy = py - from.y[jdx];
			double r2 = dx * dx + dy * dy;
			h = fmax(h, r2);
			Hxx += dx * dx; Hxy += dx * dy;
			Hyx += dy * dx; Hyy += dy * dy;
		}
		h = sqrt(h);
		h /= 2;
		to.h[i] = h;
		glm::dmat2x2 V, D;
		eigen2(glm::dmat2x2(Hxx / nc, Hyx / nc, Hxy / nc, Hyy / nc), V, D);
		double a = 1.6651 * sqrt(D[0][0]);
		double b = 1.6651 * sqrt(D[1][1]);
		double phi = atan2(V[0][1], V[0][0]);
		unsigned nbh_iter = 0;
		for (unsigned j = 0; j < nc; j++) {
			unsigned jdx = to.cand[(size_t)i * MAX_NBH + j];
			double xc = from.x[jdx] - px, yc = from.y[jdx] - py;
			double left = ((cos(phi) * xc + sin(phi) * yc) / a);
			double right = ((sin(phi) * xc - cos(phi) * yc) / b);
			if (left * left + right * right <= 1) to.nbh[(size_t)i * MAX_NBH + nbh_iter++] = jdx;
		}
		if (!(nbh_iter > 0)) throw Fail{"nbh_ellipse: no neighbours (neighbor_ellipse.h:125)"};
		to.num_nbh[i] = nbh_iter;
	}
}

// -------------------------------------------------------------------- actions
struct Ctx {
	const Case* c;
	Consts k;
	double time = 0.;
};

typedef void (*ActFn)(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet* Q);

// riemann_update_integration_weights, riemann_integration.h:28-33
void a_riemann(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	for (unsigned i = 0; i < P.n; i++) { unsigned s = perm[i]; P.qw[s] = P.m[s] / P.rho[s]; }
}
// do_material_eos, material.h:37-44
void eos_range(PSet& P, const std::vector<unsigned>& perm, double rho0, double K) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned s = perm[i];
		double c0 = sqrt(K / rho0);
		P.p[s] = c0 * c0 * (P.rho[s] - rho0);
	}
}
void a_eos(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) { eos_range(P, perm, c.k.rho0, c.k.K()); }
// stress_angle + correctors_mghn_artificial_stress, correctors.h:37-81
void a_art_stress(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double eps = c.c->mghn_eps;
	for (unsigned i = 0; i < P.n; i++) {
		unsigned s = perm[i];
		double rhoi = P.rho[s];
		double sxx = P.Sxx[s] - P.p[s];
		double syy = P.Syy[s] - P.p[s];
		double sxy = P.Sxy[s];
		double numer = 2. * sxy;
		double denom = sxx - syy + 0.;
		double theta = 0.5 * atan2(numer, denom);
		double cos_theta = cos(theta), sin_theta = sin(theta);
		double cos_theta2 = cos_theta * cos_theta, sin_theta2 = sin_theta * sin_theta;
		double rot_sxx = cos_theta2 * sxx + 2.0 * cos_theta * sin_theta * sxy + sin_theta2 * syy;
		double rot_syy = sin_theta2 * sxx - 2.0 * cos_theta * sin_theta * sxy + cos_theta2 * syy;
		double rot_rxx = 0., rot_ryy = 0.;
		if (rot_sxx > 0) rot_rxx = -eps * rot_sxx / (rhoi * rhoi);
		if (rot_syy > 0) rot_ryy = -eps * rot_syy / (rhoi * rhoi);
		P.Rxx[s] = cos_theta2 * rot_rxx + sin_theta2 * rot_ryy;
		P.Rxy[s] = cos_theta * sin_theta * (rot_rxx - rot_ryy);
		P.Ryy[s] = sin_theta2 * rot_rxx + cos_theta2 * rot_ryy;
	}
}
// derive_stress_monaghan, derivatives.h:378-443
void a_stress_monaghan(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double wdeltap = c.c->wdeltap, corr_exp = c.c->corr_exp;
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double Sxxi = P.Sxx[si] - P.p[si], Sxyi = P.Sxy[si], Syyi = P.Syy[si] - P.p[si];
		double Rxxi = P.Rxx[si], Rxyi = P.Rxy[si], Ryyi = P.Ryy[si];
		double rhoi = P.rho[si];
		double rhoi21 = 1. / (rhoi * rhoi);
		double Sxx_x = 0., Sxy_y = 0., Sxy_x = 0., Syy_y = 0.;
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			double ww = P.w[o], wx = P.w_x[o], wy = P.w_y[o];
			double Sxxj = P.Sxx[sj] - P.p[sj], Sxyj = P.Sxy[sj], Syyj = P.Syy[sj] - P.p[sj];
			double Rxxj = P.Rxx[sj], Rxyj = P.Rxy[sj], Ryyj = P.Ryy[sj];
			double mj = P.m[sj];
			double rhoj21 = 1. / (P.rho[sj] * P.rho[sj]);
			double Rxx = 0, Rxy = 0., Ryy = 0.;
			if (wdeltap > 0) {
				double fab = ww / wdeltap;
				fab = pow(fab, corr_exp);
				Rxx = fab * (Rxxi + Rxxj);
				Rxy = fab * (Rxyi + Rxyj);
				Ryy = fab * (Ryyi + Ryyj);
			}
			Sxx_x += mj * (Sxxi * rhoi21 + Sxxj * rhoj21 + Rxx) * wx;
			Sxy_y += mj * (Sxyi * rhoi21 + Sxyj * rhoj21 + Rxy) * wy;
			Sxy_x += mj * (Sxyi * rhoi21 + Sxyj * rhoj21 + Rxy) * wx;
			Syy_y += mj * (Syyi * rhoi21 + Syyj * rhoj21 + Ryy) * wy;
		}
		P.Sxx_x[si] = Sxx_x * rhoi;
		P.Sxy_y[si] = Sxy_y * rhoi;
		P.Sxy_x[si] = Sxy_x * rhoi;
		P.Syy_y[si] = Syy_y * rhoi;
	}
}
// derive_velocity (derivatives.h:32-66) and derive_velocity_tl (:483-519): the
// same gradient, written into vx_x.. or Fdot..
void vel_grad(PSet& P, const std::vector<unsigned>& perm, bool tl) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double vxi = P.vx[si], vyi = P.vy[si];
		double a = 0., b = 0., cc = 0., d = 0.;
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			double vxj = P.vx[sj], vyj = P.vy[sj];
			double qwj = P.qw[sj];
			a += (vxj - vxi) * P.w_x[o] * qwj;
			b += (vxj - vxi) * P.w_y[o] * qwj;
			cc += (vyj - vyi) * P.w_x[o] * qwj;
			d += (vyj - vyi) * P.w_y[o] * qwj;
		}
		if (tl) { P.Fdxx[si] = a; P.Fdxy[si] = b; P.Fdyx[si] = cc; P.Fdyy[si] = d; }
		else { P.vx_x[si] = a; P.vx_y[si] = b; P.vy_x[si] = cc; P.vy_y[si] = d; }
	}
}
void a_derive_velocity(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) { vel_grad(P, perm, false); }
void a_derive_velocity_tl(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) { vel_grad(P, perm, true); }
// correctors_mghn_artificial_viscosity, correctors.h:83-137
void a_art_visc(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double alpha = c.c->alpha, beta = c.c->beta, eta = c.c->eta;
	double K = c.k.K();
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double xi = P.x[si], yi = P.y[si], vxi = P.vx[si], vyi = P.vy[si], hi = P.h[si], rhoi = P.rho[si];
		double ci = sqrt(K / rhoi);
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			double xj = P.x[sj], yj = P.y[sj], vxj = P.vx[sj], vyj = P.vy[sj], hj = P.h[sj], mj = P.m[sj], rhoj = P.rho[sj];
			double cj = sqrt(K / rhoj);
			double vijx = vxi - vxj, vijy = vyi - vyj;
			double xij = xi - xj, yij = yi - yj;
			double vijposij = vijx * xij + vijy * yij;
			if (vijposij >= 0.) continue;
			double cij = 0.5 * (ci + cj);
			double hij = 0.5 * (hi + hj);
			double rhoij = 0.5 * (rhoi + rhoj);
			double r2ij = xij * xij + yij * yij;
			double muij = (hij * vijposij) / (r2ij + eta * eta * hij * hij);
			double piij = (-alpha * cij * muij + beta * muij * muij) / rhoij;
			P.vx_t[si] += -mj * piij * P.w_x[o];
			P.vy_t[si] += -mj * piij * P.w_y[o];
		}
	}
}
// correctors_xsph, correctors.h:139-169
void a_xsph(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double eps = c.c->xsph_eps;
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double vxi = P.vx[si], vyi = P.vy[si], rhoi = P.rho[si];
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			double vijx = vxi - P.vx[sj], vijy = vyi - P.vy[sj];
			double rhoij = 0.5 * (rhoi + P.rho[sj]);
			double fac = -eps * P.w[o] * P.m[si] / rhoij;
			P.x_t[si] += fac * vijx;
			P.y_t[si] += fac * vijy;
		}
	}
}
// do_material_stress_rate_jaumann, material.h:66-84
void jaumann_range(PSet& P, const std::vector<unsigned>& perm, double G) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned s = perm[i];
		glm::dmat2x2 epsdot(P.vx_x[s], 0.5 * (P.vx_y[s] + P.vy_x[s]), 0.5 * (P.vx_y[s] + P.vy_x[s]), P.vy_y[s]);
		glm::dmat2x2 omega(0., 0.5 * (P.vy_x[s] - P.vx_y[s]), 0.5 * (P.vx_y[s] - P.vy_x[s]), 0.);
		glm::dmat2x2 S(P.Sxx[s], P.Sxy[s], P.Sxy[s], P.Syy[s]);
		glm::dmat2x2 I(1.);
		double trace_epsdot = epsdot[0][0] + epsdot[1][1];
		glm::dmat2x2 S_t = 2 * G * (epsdot - 1. / 3. * trace_epsdot * I) - S * omega + omega * S;
		P.Sxx_t[s] += S_t[0][0];
		P.Sxy_t[s] += S_t[0][1];
		P.Syy_t[s] += S_t[1][1];
	}
}
void a_jaumann(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) { jaumann_range(P, perm, c.k.G()); }
// do_contmech_continuity, cont_mech.h:108-120
void continuity_range(PSet& P, const std::vector<unsigned>& perm) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned s = perm[i];
		P.rho_t[s] -= P.rho[s] * (P.vx_x[s] + P.vy_y[s]);
	}
}
void a_continuity(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) { continuity_range(P, perm); }
// contmech_momentum_ul, cont_mech.h:32-49
void a_momentum_ul(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		unsigned s = perm[i];
		double rho = P.rho[s];
		P.vx_t[s] += 1. / rho * (P.Sxx_x[s] + P.Sxy_y[s]) + P.fcx[s] / P.m[s];
		P.vy_t[s] += 1. / rho * (P.Sxy_x[s] + P.Syy_y[s]) + P.fcy[s] / P.m[s];
	}
}
// contmech_advection, cont_mech.h:134-142
void a_advection(Ctx&, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	for (unsigned i = 0; i < P.n; i++) { unsigned s = perm[i]; P.x_t[s] += P.vx[s]; P.y_t[s] += P.vy[s]; }
}
// derive_displacement, derivatives.h:101-149 (also the _weak variant :152-200
// with Gauss points as i and particles as j)
void disp_grad(PSet& Pi, const PSet& Pj) {
	for (unsigned i = 0; i < Pi.n; i++) {
		double uxi = Pi.x[i] - Pi.X[i], uyi = Pi.y[i] - Pi.Y[i];
		double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
		for (unsigned j = 0; j < Pi.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Pi.nbh[o];
			double uxj = Pj.x[jdx] - Pj.X[jdx], uyj = Pj.y[jdx] - Pj.Y[jdx];
			double qwj = Pj.qw[jdx];
			Hxx += (uxj - uxi) * Pi.w_x[o] * qwj;
			Hxy += (uxj - uxi) * Pi.w_y[o] * qwj;
			Hyx += (uyj - uyi) * Pi.w_x[o] * qwj;
			Hyy += (uyj - uyi) * Pi.w_y[o] * qwj;
		}
		Pi.Hxx[i] = Hxx; Pi.Hxy[i] = Hxy; Pi.Hyx[i] = Hyx; Pi.Hyy[i] = Hyy;
	}
}
void a_derive_displacement(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) { disp_grad(P, P); }
// do_material_compute_stress_green_stvenant, material.h:132-146
void green_stvenant_range(PSet& P, double E, double nu) {
	double D = E / (1 - nu * nu);
	for (unsigned i = 0; i < P.n; i++) {
		glm::dmat2x2 F(P.Hxx[i] + 1., P.Hyx[i], P.Hxy[i], P.Hyy[i] + 1.);
		glm::dmat2x2 C = glm::transpose(F) * F;
		glm::dmat2x2 Esv = 0.5 * (C - glm::dmat2x2(1.));
		P.Sxx[i] = D * (Esv[0][0] + nu * Esv[1][1]);
		P.Syy[i] = D * (Esv[0][0] * nu + Esv[1][1]);
		P.Sxy[i] = D * (1 - nu) * Esv[1][0];
	}
}
void a_green_stvenant(Ctx& c, PSet& P, const std::vector<unsigned>&, PSet*) { green_stvenant_range(P, c.c->E, c.c->nu); }
// do_contmech_cauchy_to_nominal, cont_mech.h:154-169
void cauchy_to_nominal_range(PSet& P) {
	for (unsigned i = 0; i < P.n; i++) {
		glm::dmat2x2 F(P.Hxx[i] + 1, P.Hyx[i], P.Hxy[i], P.Hyy[i] + 1);
		double J = glm::determinant(F);
		glm::dmat2x2 sigma(P.Sxx[i] - P.p[i], P.Sxy[i], P.Sxy[i], P.Syy[i] - P.p[i]);
		glm::dmat2x2 Finv = glm::inverse(F);
		glm::dmat2x2 Pm = J * Finv * sigma;
		P.Pxx[i] = Pm[0][0]; P.Pxy[i] = Pm[1][0]; P.Pyx[i] = Pm[0][1]; P.Pyy[i] = Pm[1][1];
	}
}
void a_cauchy_to_nominal(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) { cauchy_to_nominal_range(P); }
// derive_stress_tl, derivatives.h:331-376
void a_stress_tl(Ctx& c, PSet& P, const std::vector<unsigned>&, PSet*) {
	double rho0 = c.k.rho0;
	for (unsigned i = 0; i < P.n; i++) {
		double Pxxi = P.Pxx[i], Pxyi = P.Pxy[i], Pyxi = P.Pyx[i], Pyyi = P.Pyy[i];
		double rhoi21 = 1. / (rho0 * rho0);
		double Pxx_x = 0., Pyx_y = 0., Pxy_x = 0., Pyy_y = 0.;
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			double mj = P.m[jdx];
			double rhoj21 = 1. / (rho0 * rho0);
			Pxx_x += mj * (Pxxi * rhoi21 + P.Pxx[jdx] * rhoj21) * P.w_x[o] * rho0;
			Pyx_y += mj * (Pyxi * rhoi21 + P.Pyx[jdx] * rhoj21) * P.w_y[o] * rho0;
			Pxy_x += mj * (Pxyi * rhoi21 + P.Pxy[jdx] * rhoj21) * P.w_x[o] * rho0;
			Pyy_y += mj * (Pyyi * rhoi21 + P.Pyy[jdx] * rhoj21) * P.w_y[o] * rho0;
		}
		P.Pxx_x[i] = Pxx_x; P.Pyx_y[i] = Pyx_y; P.Pxy_x[i] = Pxy_x; P.Pyy_y[i] = Pyy_y;
	}
}
// contmech_momentum_tl, cont_mech.h:70-87
void a_momentum_tl(Ctx& c, PSet& P, const std::vector<unsigned>&, PSet*) {
	double rho0 = c.k.rho0;
	for (unsigned i = 0; i < P.n; i++) {
		P.vx_t[i] += 1. / rho0 * (P.Pxx_x[i] + P.Pyx_y[i]) + P.fcx[i] / P.m[i];
		P.vy_t[i] += 1. / rho0 * (P.Pxy_x[i] + P.Pyy_y[i]) + P.fcy[i] / P.m[i];
	}
}
// contmech_velocity_gradient_tl(_gp), cont_mech.h:171-203
void vel_grad_tl_range(PSet& P) {
	for (unsigned i = 0; i < P.n; i++) {
		glm::dmat2x2 F(P.Hxx[i] + 1., P.Hyx[i], P.Hxy[i], P.Hyy[i] + 1.);
		glm::dmat2x2 Fdot(P.Fdxx[i], P.Fdyx[i], P.Fdxy[i], P.Fdyy[i]);
		glm::dmat2x2 Finv = glm::inverse(F);
		glm::dmat2x2 L = Fdot * Finv;
		P.vx_x[i] = L[0][0]; P.vx_y[i] = L[1][0]; P.vy_x[i] = L[0][1]; P.vy_y[i] = L[1][1];
	}
}
void a_vel_grad_tl(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) { vel_grad_tl_range(P); }

// --- Gauss-point (weak form) actions; Q = the quad points
void a_disp_weak(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) { disp_grad(*Q, P); }
// derive_velocity_tl_weak, derivatives.h:445-481
void a_vel_tl_weak(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < Q->n; i++) {
		double vxi = Q->vx[i], vyi = Q->vy[i];
		double a = 0., b = 0., cc = 0., d = 0.;
		for (unsigned j = 0; j < Q->num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Q->nbh[o];
			double vxj = P.vx[jdx], vyj = P.vy[jdx], qwj = P.qw[jdx];
			a += (vxj - vxi) * Q->w_x[o] * qwj;
			b += (vxj - vxi) * Q->w_y[o] * qwj;
			cc += (vyj - vyi) * Q->w_x[o] * qwj;
			d += (vyj - vyi) * Q->w_y[o] * qwj;
		}
		Q->Fdxx[i] = a; Q->Fdxy[i] = b; Q->Fdyx[i] = cc; Q->Fdyy[i] = d;
	}
}
std::vector<unsigned> ident(unsigned n) {
	std::vector<unsigned> v(n);
	for (unsigned i = 0; i < n; i++) v[i] = i;
	return v;
}
void a_vel_grad_tl_gp(Ctx&, PSet&, const std::vector<unsigned>&, PSet* Q) { vel_grad_tl_range(*Q); }
void a_continuity_gp(Ctx&, PSet&, const std::vector<unsigned>&, PSet* Q) { continuity_range(*Q, ident(Q->n)); }
void a_eos_gp(Ctx& c, PSet&, const std::vector<unsigned>&, PSet* Q) { eos_range(*Q, ident(Q->n), c.k.rho0, c.k.K()); }
void a_jaumann_gp(Ctx& c, PSet&, const std::vector<unsigned>&, PSet* Q) { jaumann_range(*Q, ident(Q->n), c.k.G()); }
void a_c2n_gp(Ctx&, PSet&, const std::vector<unsigned>&, PSet* Q) { cauchy_to_nominal_range(*Q); }
// derive_stress_weak_tl, derivatives.h:260-294 (scatter from Gauss points to particles)
void a_stress_weak_tl(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < P.n; i++) { P.Pxx_x[i] = 0.; P.Pyx_y[i] = 0.; P.Pxy_x[i] = 0.; P.Pyy_y[i] = 0.; }
	for (unsigned i = 0; i < Q->n; i++) {
		double Pxxi = Q->Pxx[i], Pxyi = Q->Pxy[i], Pyxi = Q->Pyx[i], Pyyi = Q->Pyy[i];
		double quad_weight = Q->qw[i];
		for (unsigned j = 0; j < Q->num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Q->nbh[o];
			double vol_node = P.qw[jdx];
			P.Pxx_x[jdx] -= Pxxi * Q->w_x[o] * quad_weight * vol_node;
			P.Pyx_y[jdx] -= Pyxi * Q->w_y[o] * quad_weight * vol_node;
			P.Pxy_x[jdx] -= Pxyi * Q->w_x[o] * quad_weight * vol_node;
			P.Pyy_y[jdx] -= Pyyi * Q->w_y[o] * quad_weight * vol_node;
		}
	}
}
// contmech_momentum_tl_weak, cont_mech.h:89-106
void a_momentum_tl_weak(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		double m = P.m[i];
		P.vx_t[i] += 1. / m * (P.Pxx_x[i] + P.Pyx_y[i]) + P.fcx[i] / P.m[i];
		P.vy_t[i] += 1. / m * (P.Pxy_x[i] + P.Pyy_y[i]) + P.fcy[i] / P.m[i];
	}
}

// --- particle_corotational (corotational.h, derivatives.h:202-258,521-588, material.h:103-130)
// corotational_anisotropy_tensor, corotational.h:31-82: the rotation of the neighbourhood
void a_corot_aniso(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		double Xi = P.X[i], Yi = P.Y[i], xi = P.x[i], yi = P.y[i];
		double Axx = 0., Axy = 0., Ayx = 0., Ayy = 0.;
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			double w = P.w[o];
			double mj = P.m[jdx];
			double xji = P.x[jdx] - xi, yji = P.y[jdx] - yi;
			double Xji = P.X[jdx] - Xi, Yji = P.Y[jdx] - Yi;
			Axx += xji * Xji * mj * w;
			Axy += xji * Yji * mj * w;
			Ayx += yji * Xji * mj * w;
			Ayy += yji * Yji * mj * w;
		}
		double x = Axx + Ayy;
		double y = Ayx - Axy;
		double theta = atan2(y, x);
		P.Rxx[i] = cos(theta);
		P.Rxy[i] = -sin(theta);
		P.Ryx[i] = sin(theta);
		P.Ryy[i] = cos(theta);
	}
}
// derive_displacement_corotational, derivatives.h:202-258: displacement in the rotated frame
void a_disp_corot(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		double Hxx = 0., Hxy = 0., Hyx = 0., Hyy = 0.;
		double xi = P.x[i], yi = P.y[i], Xi = P.X[i], Yi = P.Y[i];
		double Rixx_inv = P.Rxx[i], Rixy_inv = P.Ryx[i], Riyx_inv = P.Rxy[i], Riyy_inv = P.Ryy[i];
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			double quad_weight = P.qw[jdx];
			double xji = P.x[jdx] - xi, yji = P.y[jdx] - yi;
			double Xji = P.X[jdx] - Xi, Yji = P.Y[jdx] - Yi;
			double uxji = Rixx_inv * xji + Rixy_inv * yji - Xji;
			double uyji = Riyx_inv * xji + Riyy_inv * yji - Yji;
			Hxx += uxji * P.w_x[o] * quad_weight;
			Hxy += uxji * P.w_y[o] * quad_weight;
			Hyx += uyji * P.w_x[o] * quad_weight;
			Hyy += uyji * P.w_y[o] * quad_weight;
		}
		P.Hxx[i] = Hxx; P.Hxy[i] = Hxy; P.Hyx[i] = Hyx; P.Hyy[i] = Hyy;
	}
}
// do_material_compute_stress_cauchy_green, material.h:103-114 (small-strain Cauchy-Green)
void a_cauchy_green(Ctx& c, PSet& P, const std::vector<unsigned>&, PSet*) {
	double E = c.c->E, nu = c.c->nu;
	double D = E / (1 - nu * nu);
	for (unsigned i = 0; i < P.n; i++) {
		glm::dmat2x2 F(P.Hxx[i] + 1., P.Hyx[i], P.Hxy[i], P.Hyy[i] + 1.);
		glm::dmat2x2 Ecg = 0.5 * (F + glm::transpose(F)) - glm::dmat2x2(1.);
		P.Sxx[i] = D * (Ecg[0][0] + nu * Ecg[1][1]);
		P.Syy[i] = D * (Ecg[0][0] * nu + Ecg[1][1]);
		P.Sxy[i] = D * (1 - nu) * Ecg[0][1];
	}
}
// derive_stress_corotational, derivatives.h:521-588: pair forces rotated back, then fc/m
void a_stress_corot(Ctx& c, PSet& P, const std::vector<unsigned>&, PSet*) {
	double rho0 = c.k.rho0;
	for (unsigned i = 0; i < P.n; i++) {
		double Pxxi = P.Pxx[i], Pxyi = P.Pxy[i], Pyxi = P.Pyx[i], Pyyi = P.Pyy[i];
		double Rxxi = P.Rxx[i], Rxyi = P.Rxy[i], Ryxi = P.Ryx[i], Ryyi = P.Ryy[i];
		double rhoi21 = 1. / (rho0 * rho0);
		double vx_t = 0., vy_t = 0.;
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			double Pxxj = P.Pxx[jdx], Pxyj = P.Pxy[jdx], Pyxj = P.Pyx[jdx], Pyyj = P.Pyy[jdx];
			double Rxxj = P.Rxx[jdx], Rxyj = P.Rxy[jdx], Ryxj = P.Ryx[jdx], Ryyj = P.Ryy[jdx];
			double mj = P.m[jdx];
			double rhoj21 = 1. / (rho0 * rho0);
			double wx = P.w_x[o], wy = P.w_y[o];
			double aijx = mj * ((Pxxi * rhoi21 + Pxxj * rhoj21) * wx + (Pxyi * rhoi21 + Pxyj * rhoj21) * wy);
			double aijy = mj * ((Pyxi * rhoi21 + Pyxj * rhoj21) * wx + (Pyyi * rhoi21 + Pyyj * rhoj21) * wy);
			double ajix = -aijx;
			double ajiy = -aijy;
			double aijxprime = aijx * Rxxi + aijy * Rxyi;
			double aijyprime = aijx * Ryxi + aijy * Ryyi;
			double ajixprime = ajix * Rxxj + ajiy * Rxyj;
			double ajiyprime = ajix * Ryxj + ajiy * Ryyj;
			vx_t += 0.5 * (aijxprime - ajixprime);
			vy_t += 0.5 * (aijyprime - ajiyprime);
		}
		P.vx_t[i] = vx_t;
		P.vy_t[i] = vy_t;
	}
	for (unsigned i = 0; i < P.n; i++) {
		P.vx_t[i] += P.fcx[i] / P.m[i];
		P.vy_t[i] += P.fcy[i] / P.m[i];
	}
}

// godunov_get_trafo, godunov.h:56-84: the pair's unit direction R = (x_j - x_i)/|.|
// and its normal S, the stresses projected on R and the velocities, all turned into
// the (R, S) frame.  The frame matrix is built as a single-precision glm::mat2x2
// (godunov.h:73), so it holds the float roundings of R and S.  The stress matrix
// subtracts the pressure from Sxx only (godunov.h:68-69).
struct GTrafo {
	glm::dmat2x2 l;
	glm::dvec2 siR, sjR, vi, vj;
};
GTrafo godunov_trafo(const PSet& P, unsigned si, unsigned sj) {
	double Rx = P.x[sj] - P.x[si];
	double Ry = P.y[sj] - P.y[si];
	double Sx = Ry, Sy = -Rx;
	glm::dvec2 R = glm::normalize(glm::dvec2(Rx, Ry));
	glm::dvec2 S = glm::normalize(glm::dvec2(Sx, Sy));
	glm::dmat2x2 sig_i(P.Sxx[si] - P.p[si], P.Sxy[si], P.Sxy[si], P.Syy[si]);
	glm::dmat2x2 sig_j(P.Sxx[sj] - P.p[sj], P.Sxy[sj], P.Sxy[sj], P.Syy[sj]);
	GTrafo t;
	t.l = glm::mat2x2(R, S);
	glm::dvec2 siR = sig_i * R, sjR = sig_j * R;
	t.siR = t.l * siR;
	t.sjR = t.l * sjR;
	t.vi = t.l * glm::dvec2(P.vx[si], P.vy[si]);
	t.vj = t.l * glm::dvec2(P.vx[sj], P.vy[sj]);
	return t;
}
// godunov_momentum, godunov.h:86-142 (Parshikov-Medin acoustic Riemann solution per
// pair; the second component uses sigma_j twice, godunov.h:116, as written)
void a_godunov_momentum(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double K = c.k.K();
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double ci = sqrt(K / P.rho[si]);
		double rhoi = P.rho[si];
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			if (P.idx[si] == P.idx[sj]) continue;
			GTrafo t = godunov_trafo(P, si, sj);
			double cj = sqrt(K / P.rho[sj]);
			double rhoj = P.rho[sj];
			double qw = P.qw[sj];
			glm::dvec2 SRs;
			double frac = 1. / (rhoi * ci + rhoj * cj);
			SRs[0] = frac * (t.sjR[0] * rhoi * ci + t.siR[0] * rhoj * cj + rhoi * ci * rhoj * cj * (t.vj[0] - t.vi[0]));
			SRs[1] = frac * (t.sjR[1] * rhoi * ci + t.sjR[1] * rhoj * cj + rhoi * ci * rhoj * cj * (t.vj[1] - t.vi[1]));
			glm::dvec2 SR = glm::transpose(t.l) * SRs;
			double rx = P.x[sj] - P.x[si];
			double ry = P.y[sj] - P.y[si];
			double mag_r = sqrt(rx * rx + ry * ry);
			if (fabs(rx) > 0.) P.vx_t[si] += 2. / rhoi * P.w_x[o] * mag_r / rx * SR[0] * qw;
			if (fabs(ry) > 0.) P.vy_t[si] += 2. / rhoi * P.w_y[o] * mag_r / ry * SR[1] * qw;
		}
	}
	for (unsigned i = 0; i < P.n; i++) {
		P.vx_t[i] += P.fcx[i] / P.m[i];
		P.vy_t[i] += P.fcy[i] / P.m[i];
	}
}
// godunov_continuity, godunov.h:144-187, with riemann_solver_acoustic (:41-54) inline
void a_godunov_continuity(Ctx& c, PSet& P, const std::vector<unsigned>& perm, PSet*) {
	double K = c.k.K();
	for (unsigned i = 0; i < P.n; i++) {
		unsigned si = perm[i];
		double xi = P.x[si], yi = P.y[si], rhoi = P.rho[si];
		double rho_t = 0.;
		for (unsigned j = 0; j < P.num_nbh[si]; j++) {
			size_t o = (size_t)si * MAX_NBH + j;
			unsigned sj = perm[P.nbh[o]];
			if (P.idx[si] == P.idx[sj]) continue;
			double dx = xi - P.x[sj], dy = yi - P.y[sj];
			double mag_r = sqrt(dx * dx + dy * dy);
			double nx = dx / mag_r, ny = dy / mag_r;
			double vir = P.vx[si] * nx + P.vy[si] * ny;
			double vjr = P.vx[sj] * nx + P.vy[sj] * ny;
			double rhol = P.rho[si], rhor = P.rho[sj], pl = P.p[si], pr = P.p[sj];
			double csl = sqrt(K / rhol), csr = sqrt(K / rhor);
			double frac = 1. / (rhol * csl + rhor * csr);
			double ustar = frac * (vir * rhol * csl + vjr * rhor * csr - pl + pr);
			rho_t += 2 * rhoi * (vir - ustar) * (P.w_x[o] * nx + P.w_y[o] * ny) * P.qw[sj];
		}
		P.rho_t[si] = rho_t;
	}
}
// potential_comp_elastic_potential, potential.h:33-83: pair forces from the elastic
// potential, f_ij = -2 V_i F_i S_i grad W_ij, with the reverse pair's gradient for f_ji
void a_potential(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		glm::dmat2x2 Ji(P.Hxx[i] + 1., P.Hyx[i], P.Hxy[i], P.Hyy[i] + 1.);
		glm::dmat2x2 Si(P.Sxx[i], P.Sxy[i], P.Sxy[i], P.Syy[i]);
		double voli = P.qw[i];
		glm::dmat2x2 Fei = -2 * voli * Ji * Si;
		double vx_t = 0., vy_t = 0.;
		for (unsigned j = 0; j < P.num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = P.nbh[o];
			glm::dvec2 fij = Fei * glm::dvec2(P.w_x[o], P.w_y[o]);
			glm::dmat2x2 Jj(P.Hxx[jdx] + 1., P.Hyx[jdx], P.Hxy[jdx], P.Hyy[jdx] + 1.);
			glm::dmat2x2 Sj(P.Sxx[jdx], P.Sxy[jdx], P.Sxy[jdx], P.Syy[jdx]);
			double volj = P.qw[jdx];
			glm::dmat2x2 Fej = -2 * volj * Jj * Sj;
			glm::dvec2 fji = Fej * glm::dvec2(P.wji_x[o], P.wji_y[o]);
			vx_t += 0.5 * (fji[0] - fij[0]) / P.m[i];
			vy_t += 0.5 * (fji[1] - fij[1]) / P.m[i];
		}
		P.vx_t[i] = vx_t;
		P.vy_t[i] = vy_t;
	}
	for (unsigned i = 0; i < P.n; i++) {
		P.vx_t[i] += P.fcx[i] / P.m[i];
		P.vy_t[i] += P.fcy[i] / P.m[i];
	}
}

// riemann_update_integration_weights_gp, riemann_integration.h:21-26
void a_riemann_gp(Ctx&, PSet&, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < Q->n; i++) Q->qw[i] = Q->m[i] / Q->rho[i];
}
// derive_stress_weak_ul, derivatives.h:296-329: each stress point scatters its stress
// times the shape-function gradient onto its particle neighbours, ascending
void a_stress_weak_ul(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < P.n; i++) { P.Sxx_x[i] = 0.; P.Sxy_y[i] = 0.; P.Sxy_x[i] = 0.; P.Syy_y[i] = 0.; }
	for (unsigned i = 0; i < Q->n; i++) {
		double Sxxi = Q->Sxx[i] - Q->p[i], Sxyi = Q->Sxy[i], Syyi = Q->Syy[i] - Q->p[i];
		double qw = Q->qw[i];
		for (unsigned j = 0; j < Q->num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Q->nbh[o];
			double vol_node = P.qw[jdx];
			P.Sxx_x[jdx] -= Sxxi * Q->w_x[o] * qw * vol_node;
			P.Sxy_y[jdx] -= Sxyi * Q->w_y[o] * qw * vol_node;
			P.Sxy_x[jdx] -= Sxyi * Q->w_x[o] * qw * vol_node;
			P.Syy_y[jdx] -= Syyi * Q->w_y[o] * qw * vol_node;
		}
	}
}
// derive_velocity_weak, derivatives.h:68-99: stress-point velocity gradients
void a_vel_weak(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < Q->n; i++) {
		double vx_x = 0., vx_y = 0., vy_x = 0., vy_y = 0.;
		for (unsigned j = 0; j < Q->num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Q->nbh[o];
			double vxj = P.vx[jdx], vyj = P.vy[jdx], qw = P.qw[jdx];
			vx_x += vxj * Q->w_x[o] * qw;
			vx_y += vxj * Q->w_y[o] * qw;
			vy_x += vyj * Q->w_x[o] * qw;
			vy_y += vyj * Q->w_y[o] * qw;
		}
		Q->vx_x[i] = vx_x; Q->vx_y[i] = vx_y; Q->vy_x[i] = vy_x; Q->vy_y[i] = vy_y;
	}
}
// contmech_momentum_ul_weak, cont_mech.h:51-68
void a_momentum_ul_weak(Ctx&, PSet& P, const std::vector<unsigned>&, PSet*) {
	for (unsigned i = 0; i < P.n; i++) {
		double m = P.m[i];
		P.vx_t[i] += 1. / m * (P.Sxx_x[i] + P.Sxy_y[i]) + P.fcx[i] / P.m[i];
		P.vy_t[i] += 1. / m * (P.Sxy_x[i] + P.Syy_y[i]) + P.fcy[i] / P.m[i];
	}
}
// interpolation_interpolate_velocity, interpolation.h:32-59
void a_interp_vel(Ctx&, PSet& P, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < Q->n; i++) {
		double vxi = 0., vyi = 0.;
		for (unsigned j = 0; j < Q->num_nbh[i]; j++) {
			size_t o = (size_t)i * MAX_NBH + j;
			unsigned jdx = Q->nbh[o];
			vxi += P.vx[jdx] * Q->w[o] * P.qw[jdx];
			vyi += P.vy[jdx] * Q->w[o] * P.qw[jdx];
		}
		Q->vx[i] = vxi;
		Q->vy[i] = vyi;
	}
}
// contmech_advection_gp, cont_mech.h:144-152
void a_advection_gp(Ctx&, PSet&, const std::vector<unsigned>&, PSet* Q) {
	for (unsigned i = 0; i < Q->n; i++) { Q->x_t[i] += Q->vx[i]; Q->y_t[i] += Q->vy[i]; }
}

ActFn action_fn(uint32_t a) {
	switch (a) {
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS: return a_riemann;
	case MATERIAL_EOS: return a_eos;
	case CORRECTORS_MGHN_ARTIFICIAL_STRESS: return a_art_stress;
	case DERIVE_STRESS_MONAGHAN: return a_stress_monaghan;
	case DERIVE_VELOCITY: return a_derive_velocity;
	case CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY: return a_art_visc;
	case CORRECTORS_XSPH: return a_xsph;
	case MATERIAL_STRESS_RATE_JAUMANN: return a_jaumann;
	case CONTMECH_CONTINUITY: return a_continuity;
	case CONTMECH_MOMENTUM_UL: return a_momentum_ul;
	case CONTMECH_ADVECTION: return a_advection;
	case DERIVE_DISPLACEMENT: return a_derive_displacement;
	case MATERIAL_COMPUTE_STRESS_GREEN_STVENANT: return a_green_stvenant;
	case CONTMECH_CAUCHY_TO_NOMINAL: return a_cauchy_to_nominal;
	case DERIVE_STRESS_TL: return a_stress_tl;
	case CONTMECH_MOMENTUM_TL: return a_momentum_tl;
	case DERIVE_VELOCITY_TL: return a_derive_velocity_tl;
	case CONTMECH_VELOCITY_GRADIENT_TL: return a_vel_grad_tl;
	case DERIVE_DISPLACEMENT_WEAK: return a_disp_weak;
	case DERIVE_VELOCITY_TL_WEAK: return a_vel_tl_weak;
	case CONTMECH_VELOCITY_GRADIENT_TL_GP: return a_vel_grad_tl_gp;
	case CONTMECH_CONTINUITY_GP: return a_continuity_gp;
	case MATERIAL_EOS_GP: return a_eos_gp;
	case MATERIAL_STRESS_RATE_JAUMANN_GP: return a_jaumann_gp;
	case CONTMECH_CAUCHY_TO_NOMINAL_GP: return a_c2n_gp;
	case DERIVE_STRESS_WEAK_TL: return a_stress_weak_tl;
	case CONTMECH_MOMENTUM_TL_WEAK: return a_momentum_tl_weak;
	case COROTATIONAL_ANISOTROPY_TENSOR: return a_corot_aniso;
	case DERIVE_DISPLACEMENT_COROTATIONAL: return a_disp_corot;
	case MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN: return a_cauchy_green;
	case DERIVE_STRESS_COROTATIONAL: return a_stress_corot;
	case GODUNOV_CONTINUITY: return a_godunov_continuity;
	case GODUNOV_MOMENTUM: return a_godunov_momentum;
	case POTENTIAL_COMP_ELASTIC_POTENTIAL: return a_potential;
	case RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP: return a_riemann_gp;
	case DERIVE_STRESS_WEAK_UL: return a_stress_weak_ul;
	case DERIVE_VELOCITY_WEAK: return a_vel_weak;
	case CONTMECH_MOMENTUM_UL_WEAK: return a_momentum_ul_weak;
	case INTERPOLATION_INTERPOLATE_VELOCITY: return a_interp_vel;
	case CONTMECH_ADVECTION_GP: return a_advection_gp;
	}
	throw Fail{"unknown action id"};
}

// ------------------------------------------------------------ kd tree, hull
// kd_point and kd_tree, kd_tree.h:25-57, kd_tree.cpp:20-116
struct KdPoint {
	double x, y, nx, ny;
};
struct KdTree {
	struct Node {
		int left, right;
		KdPoint point;
	};
	std::vector<KdPoint> pts;
	std::vector<Node> nodes;
	int root = -1;
	static bool by_x(const KdPoint a, const KdPoint b) { return a.x < b.x; }
	static bool by_y(const KdPoint a, const KdPoint b) { return a.y < b.y; }
	int build(unsigned start, unsigned end, unsigned level) {
		int id = (int)nodes.size();
		nodes.push_back(Node{-1, -1, KdPoint{0, 0, 0, 0}});
		std::sort(pts.begin() + start, pts.begin() + end, (level % 2) ? by_x : by_y);
		int median = (end + start) / 2;
		nodes[id].point = pts[median];
		int left_lo = start, left_hi = median, right_lo = median + 1, right_hi = end;
		int l = (left_hi - left_lo > 0) ? build(left_lo, left_hi, level + 1) : -1;
		nodes[id].left = l;
		int r = (right_hi - right_lo > 0) ? build(right_lo, right_hi, level + 1) : -1;
		nodes[id].right = r;
		return id;
	}
	KdTree(const std::vector<KdPoint>& p) : pts(p) {
		nodes.reserve(p.size());
		root = p.empty() ? -1 : build(0, (unsigned)p.size(), 0);
	}
	void find(int cur, double qx, double qy, KdPoint* closest, double* best, unsigned level) const {
		if (cur < 0) return;
		const Node& nd = nodes[cur];
		bool left = (level % 2 && qx < nd.point.x) || (!(level % 2) && qy < nd.point.y);
		if (left) find(nd.left, qx, qy, closest, best, level + 1);
		else find(nd.right, qx, qy, closest, best, level + 1);
		double dx = qx - nd.point.x, dy = qy - nd.point.y;
		double dx2 = dx * dx, dy2 = dy * dy;
		double dist2 = dx2 + dy2;
		if (dist2 < *best) { *best = dist2; *closest = nd.point; }
		if (*best > dx2 || *best > dy2) {
			if (left) find(nd.right, qx, qy, closest, best, level + 1);
			else find(nd.left, qx, qy, closest, best, level + 1);
		}
	}
	KdPoint closest(double qx, double qy) const {
		KdPoint c{0, 0, 0, 0};
		double best = DBL_MAX;
		find(root, qx, qy, &c, &best, 0);
		return c;
	}
};

// boundary::update_normals, boundary.h:50-76
void update_normals(std::vector<KdPoint>& b) {
	unsigned nb = (unsigned)b.size();
	for (unsigned i = 0; i < nb; i++) {
		int left = ((int)i) - 1;
		int right = i + 1;
		if (left < 0) left = nb - 1;
		if (right >= (int)nb) right = 0;
		glm::dvec2 left_p(b[left].x, b[left].y), p(b[i].x, b[i].y), right_p(b[right].x, b[right].y);
		glm::dvec2 tl = left_p - p, tr = right_p - p;
		glm::dvec2 nl = glm::normalize(glm::dvec2(-tl.y, tl.x));
		glm::dvec2 nr = glm::normalize(glm::dvec2(tr.y, -tr.x));
		glm::dvec2 n = 0.5 * (nl + nr);
		b[i].nx = n.x;
		b[i].ny = n.y;
	}
}

// --------------------------------------------------------------------- bodies
// element (element.h): the ll, lr, tr, tl node indices of a bilinear quadrilateral
struct Elem {
	unsigned ll, lr, tr, tl;
};

struct Body {
	unsigned n = 0;
	PSet P, k[4];
	PSet Q, kq[4];  // Gauss points (TL_WEAK) / stress points (UL_WEAK)
	std::vector<Elem> elems;  // UL_WEAK with a gauss_int (the *_ul_fem set-ups), else empty
	unsigned gorder = 0;
	std::vector<unsigned> perm[4];
	std::vector<unsigned> hull;
	std::vector<KdPoint> bnd;
	std::vector<BC> bcs;
	Grid grid;
};

// boundary_conditions::carry_out_boundary_conditions, boundary_conditions.h:36-46,
// with the pull functors of tensile.cpp:20-42
void carry_out_bc(const Body& B, PSet& P, double t) {
	for (const BC& bc : B.bcs) {
		for (unsigned i : bc.idx) {
			if (bc.kind == BC_PULL_TL) {  // left/right_bndry_fun_tl, tensile.cpp:20-42
				P.x[i] = P.X[i] + bc.v * t;
				P.y[i] = P.Y[i];
				P.vx[i] = bc.v;
				P.vy[i] = 0.;
				P.vx_t[i] = 0.;
				P.vy_t[i] = 0.;
			} else if (bc.kind == BC_VELOCITY_UL) {  // left/right_bndry_fun_ul, tensile.cpp:44-66
				P.x_t[i] = bc.v;
				P.y_t[i] = 0.;
				P.vx[i] = bc.v;
				P.vy[i] = 0.;
				P.vx_t[i] = 0.;
				P.vy_t[i] = 0.;
			}
		}
	}
}

void update_gauss_points(PSet& Q, const std::vector<double>& nx, const std::vector<double>& ny,
                         const std::vector<Elem>& elems, unsigned order);

struct Sim {
	Case c;
	Ctx ctx;
	std::vector<Body> bodies;
	std::vector<std::vector<std::vector<unsigned>>> first_nbh;  // per body, per particle idx, neighbour idx list
	bool recorded = false;

	void record_nbh(const PSet& P, const std::vector<unsigned>& perm, unsigned b) {
		auto& L = first_nbh[b];
		L.assign(P.n, {});
		for (unsigned i = 0; i < P.n; i++) {
			unsigned si = perm[i];
			for (unsigned j = 0; j < P.num_nbh[si]; j++) L[P.idx[si]].push_back(P.idx[perm[P.nbh[(size_t)si * MAX_NBH + j]]]);
		}
	}

	// body::compute_time_derivatives: UL body.h:125-148, TL :110-123, TL weak :60-78
	void derivs(unsigned b, unsigned s) {
		Body& B = bodies[b];
		PSet& P = B.k[s];
		std::vector<unsigned>& perm = B.perm[s];
		for (unsigned i = 0; i < P.n; i++) P.reset(i);
		if (c.method == UL) {
			B.grid.update_geometry(P, perm, 2.);
			B.grid.assign_hashes(P, perm);
			std::sort(perm.begin(), perm.end(), [&P](unsigned a, unsigned bb) { return P.hash[a] < P.hash[bb]; });
			B.grid.construct_verlet_lists(P, perm, c.nbh_eps);
			precomp_sph(P, perm);
			if (!recorded && s == 0) record_nbh(P, perm, b);
			for (uint32_t a : c.actions) action_fn(a)(ctx, P, perm, nullptr);
			std::sort(perm.begin(), perm.end(), [&P](unsigned a, unsigned bb) { return P.idx[a] < P.idx[bb]; });
		} else if (c.method == TL || c.method == COROT || c.method == POTENTIAL) {
			carry_out_bc(B, P, ctx.time);
			for (uint32_t a : c.actions) action_fn(a)(ctx, P, perm, nullptr);
		} else if (c.method == UL_WEAK) {
			// body.h:80-108: this stage's neighbourhoods and shape functions, the
			// actions, then the boundary conditions
			PSet& Q = B.kq[s];
			for (unsigned i = 0; i < Q.n; i++) Q.reset(i);
			if (B.gorder) {
				update_gauss_points(Q, P.x, P.y, B.elems, B.gorder);
			} else {
				nbh_ellipse(P, P);
				nbh_ellipse(Q, P);
				precomp_rkpm(Q, P);
				precomp_rkpm(P, P);
			}
			if (!recorded && s == 0) record_nbh(P, perm, b);
			for (uint32_t a : c.actions) action_fn(a)(ctx, P, perm, &Q);
			carry_out_bc(B, P, ctx.time);
		} else {
			PSet& Q = B.kq[s];
			for (unsigned i = 0; i < Q.n; i++) Q.reset(i);
			carry_out_bc(B, P, ctx.time);
			for (uint32_t a : c.actions) action_fn(a)(ctx, P, perm, &Q);
		}
	}

	// rk4::rk_add, rk4.h:52-69
	static void rk_add(const PSet& kin, const PSet& init, PSet& kout, double dt) {
		for (unsigned i = 0; i < init.n; i++) {
			copy_into(init, i, kout, i);
			kout.x[i] += kin.x_t[i] * dt;
			kout.y[i] += kin.y_t[i] * dt;
			kout.vx[i] += kin.vx_t[i] * dt;
			kout.vy[i] += kin.vy_t[i] * dt;
			kout.rho[i] += kin.rho_t[i] * dt;
			kout.Sxx[i] += kin.Sxx_t[i] * dt;
			kout.Sxy[i] += kin.Sxy_t[i] * dt;
			kout.Syy[i] += kin.Syy_t[i] * dt;
		}
	}

	// rk4::step_strong (rk4.h:71-108) and rk4::do_step_weak + step (rk4.h:140-185,207-218)
	void step_body(unsigned b) {
		Body& B = bodies[b];
		double m_dt = c.dt;
		bool weak = c.method == TL_WEAK || c.method == UL_WEAK;
		for (unsigned i = 0; i < B.n; i++) copy_into(B.P, i, B.k[0], i);
		if (weak) for (unsigned i = 0; i < B.Q.n; i++) copy_into(B.Q, i, B.kq[0], i);
		const double fr[3] = {0.5, 0.5, 1.0};
		for (int s = 0; s < 4; s++) {
			derivs(b, s);
			if (s < 3) {
				rk_add(B.k[s], B.P, B.k[s + 1], fr[s] * m_dt);
				if (weak) rk_add(B.kq[s], B.Q, B.kq[s + 1], fr[s] * m_dt);
			}
		}
		recorded = recorded || (b + 1 == bodies.size());
		PSet& P = B.P;
		const PSet *k1 = &B.k[0], *k2 = &B.k[1], *k3 = &B.k[2], *k4 = &B.k[3];
		for (unsigned i = 0; i < B.n; i++) {
			P.x[i] += m_dt * 1. / 6. * (k1->x_t[i] + 2 * k2->x_t[i] + 2 * k3->x_t[i] + k4->x_t[i]);
			P.y[i] += m_dt * 1. / 6. * (k1->y_t[i] + 2 * k2->y_t[i] + 2 * k3->y_t[i] + k4->y_t[i]);
			P.rho[i] += m_dt * 1. / 6. * (k1->rho_t[i] + 2 * k2->rho_t[i] + 2 * k3->rho_t[i] + k4->rho_t[i]);
			P.vx[i] += m_dt * 1. / 6. * (k1->vx_t[i] + 2 * k2->vx_t[i] + 2 * k3->vx_t[i] + k4->vx_t[i]);
			P.vy[i] += m_dt * 1. / 6. * (k1->vy_t[i] + 2 * k2->vy_t[i] + 2 * k3->vy_t[i] + k4->vy_t[i]);
			if (!weak) {
				P.Sxx[i] += m_dt * 1. / 6. * (k1->Sxx_t[i] + 2 * k2->Sxx_t[i] + 2 * k3->Sxx_t[i] + k4->Sxx_t[i]);
				P.Sxy[i] += m_dt * 1. / 6. * (k1->Sxy_t[i] + 2 * k2->Sxy_t[i] + 2 * k3->Sxy_t[i] + k4->Sxy_t[i]);
				P.Syy[i] += m_dt * 1. / 6. * (k1->Syy_t[i] + 2 * k2->Syy_t[i] + 2 * k3->Syy_t[i] + k4->Syy_t[i]);
			}
		}
		if (weak) {
			PSet& Q = B.Q;
			const PSet *q1 = &B.kq[0], *q2 = &B.kq[1], *q3 = &B.kq[2], *q4 = &B.kq[3];
			for (unsigned i = 0; i < Q.n; i++) {
				Q.x[i] += m_dt * 1. / 6. * (q1->x_t[i] + 2 * q2->x_t[i] + 2 * q3->x_t[i] + q4->x_t[i]);
				Q.y[i] += m_dt * 1. / 6. * (q1->y_t[i] + 2 * q2->y_t[i] + 2 * q3->y_t[i] + q4->y_t[i]);
				Q.rho[i] += m_dt * 1. / 6. * (q1->rho_t[i] + 2 * q2->rho_t[i] + 2 * q3->rho_t[i] + q4->rho_t[i]);
				Q.Sxx[i] += m_dt * 1. / 6. * (q1->Sxx_t[i] + 2 * q2->Sxx_t[i] + 2 * q3->Sxx_t[i] + q4->Sxx_t[i]);
				Q.Sxy[i] += m_dt * 1. / 6. * (q1->Sxy_t[i] + 2 * q2->Sxy_t[i] + 2 * q3->Sxy_t[i] + q4->Sxy_t[i]);
				Q.Syy[i] += m_dt * 1. / 6. * (q1->Syy_t[i] + 2 * q2->Syy_t[i] + 2 * q3->Syy_t[i] + q4->Syy_t[i]);
			}
			ctx.time += m_dt;  // rk4.h:194 / :214
			carry_out_bc(B, P, ctx.time);
			if (c.method == UL_WEAK) {
				if (c.do_smooth) {  // rk4.h:198-204: fresh neighbourhoods and weights first
					nbh_ellipse(P, P);
					for (unsigned i = 0; i < P.n; i++) P.qw[i] = P.m[i] / P.rho[i];
					precomp_rkpm(P, P);
					smooth_vel(B);
				}
			} else if (c.do_smooth) {
				smooth_vel(B);
			}
		} else {
			carry_out_bc(B, P, ctx.time);  // rk4.h:105
			ctx.time += m_dt;              // rk4.h:107
		}
	}

	// correctors_smooth_vel, correctors.h:171-210 (on the base particles)
	void smooth_vel(Body& B) {
		PSet& P = B.P;
		std::vector<double> vsx(P.n), vsy(P.n);
		for (unsigned i = 0; i < P.n; i++) {
			double a = 0., bb = 0.;
			for (unsigned j = 0; j < P.num_nbh[i]; j++) {
				size_t o = (size_t)i * MAX_NBH + j;
				unsigned jdx = P.nbh[o];
				a += P.vx[jdx] * P.w[o] * P.qw[jdx];
				bb += P.vy[jdx] * P.w[o] * P.qw[jdx];
			}
			vsx[i] = a;
			vsy[i] = bb;
		}
		for (unsigned i = 0; i < P.n; i++) { P.vx[i] = vsx[i]; P.vy[i] = vsy[i]; }
	}

	// body::update_boundary, body.h:153-166
	void update_boundary(Body& B) {
		if (B.hull.empty()) return;
		for (unsigned i = 0; i < B.hull.size(); i++) { B.bnd[i].x = B.P.x[B.hull[i]]; B.bnd[i].y = B.P.y[B.hull[i]]; }
		update_normals(B.bnd);
	}

	// contact_apply_body_to_boundary, contact.h:36-80
	void contact(Body& master, Body& slave) {
		if (slave.hull.empty() || master.hull.empty()) return;
		double dt = c.dt;
		double dt2 = dt * dt;
		KdTree tree(master.bnd);
		const double alpha = 0.1;
		PSet& S = slave.P;
		for (unsigned i = 0; i < S.n; i++) { S.fcx[i] = 0.; S.fcy[i] = 0.; }
		for (unsigned i = 0; i < S.n; i++) {
			double qx = S.x[i], qy = S.y[i];
			KdPoint cp = tree.closest(qx, qy);
			double dx = qx - cp.x, dy = qy - cp.y;
			double pdotn = dx * cp.nx + dy * cp.ny;
			bool inside = pdotn <= 0.;
			if (!inside) continue;
			double gN_nx = cp.nx * pdotn, gN_ny = cp.ny * pdotn;
			double ms = S.m[i];
			double fcx = ms * gN_nx / dt2 * alpha;
			double fcy = ms * gN_ny / dt2 * alpha;
			S.fcx[i] = -fcx;
			S.fcy[i] = -fcy;
		}
	}

	// the step loop of main(), mfree_iwf.cpp:84-97
	void driver_step() {
		for (unsigned b = 0; b < bodies.size(); b++) {
			step_body(b);
			update_boundary(bodies[b]);
		}
		if (c.contact)
			for (unsigned i = 0; i < bodies.size(); i++)
				for (unsigned j = 0; j < bodies.size(); j++)
					if (i != j) contact(bodies[i], bodies[j]);
	}

	void setup() {
		ctx.c = &c;
		ctx.k = Consts{c.nu, c.E, c.rho0};
		bodies.resize(c.nbodies);
		first_nbh.resize(c.nbodies);
		for (unsigned b = 0; b < c.nbodies; b++) {
			Body& B = bodies[b];
			const BodyIn& in = c.bodies[b];
			B.n = in.n;
			B.P.resize(in.n);
			for (int s = 0; s < 4; s++) { B.k[s].resize(in.n); B.perm[s] = ident(in.n); }
			std::vector<double>* dst[NIN] = {&B.P.x, &B.P.y, &B.P.X, &B.P.Y, &B.P.m, &B.P.rho, &B.P.h, &B.P.qw,
			                                 &B.P.vx, &B.P.vy, &B.P.Sxx, &B.P.Sxy, &B.P.Syy};
			for (int a = 0; a < NIN; a++) *dst[a] = in.a[a];
			B.hull = in.hull;
			B.bnd.assign(B.hull.size(), KdPoint{0, 0, 0, 0});
			B.bcs = in.bcs;
			if (c.method == TL) {
				// rings.cpp:404-408 / tensile.cpp:268-269
				find_neighbors(B.P, B.P, c.nbh_h, c.nbh_eps);
				precomp_randles_libersky(B.P);
				record_nbh(B.P, ident(B.n), b);
			} else if (c.method == COROT) {
				// rings.cpp:311-315 / tensile.cpp:197-198: plain SPH weights on the set-up lists
				find_neighbors(B.P, B.P, c.nbh_h, c.nbh_eps);
				precomp_sph(B.P, ident(B.n));
				record_nbh(B.P, ident(B.n), b);
			} else if (c.method == POTENTIAL) {
				// rings.cpp:497-501 / tensile.cpp:345-346: symmetric Randles-Libersky weights
				find_neighbors(B.P, B.P, c.nbh_h, c.nbh_eps);
				precomp_randles_libersky_symmetric(B.P);
				record_nbh(B.P, ident(B.n), b);
			} else if (c.method == TL_WEAK) {
				setup_weak(B, in);
				record_nbh(B.P, ident(B.n), b);
			} else if (c.method == UL_WEAK) {
				// the stress points as given; candidates by the Manhattan search
				// (tensile.cpp:706-707, rings.cpp:900-904)
				B.Q.resize(in.ngp);
				for (int s = 0; s < 4; s++) B.kq[s].resize(in.ngp);
				std::vector<double>* gd[NIN] = {&B.Q.x, &B.Q.y, &B.Q.X, &B.Q.Y, &B.Q.m, &B.Q.rho, &B.Q.h, &B.Q.qw,
				                                &B.Q.vx, &B.Q.vy, &B.Q.Sxx, &B.Q.Sxy, &B.Q.Syy};
				for (int a = 0; a < NIN; a++) *gd[a] = in.g[a];
				if (in.ex == 1) {
					// a gauss_int replaces the ellipse (body.h:91-99): no candidates
					for (size_t e = 0; e + 3 < in.quads.size(); e += 4)
						B.elems.push_back(Elem{in.quads[e], in.quads[e + 1], in.quads[e + 2], in.quads[e + 3]});
					B.gorder = in.order;
					if ((size_t)B.gorder * B.gorder * B.elems.size() != in.ngp) throw Fail{"element map and stress points differ"};
				} else {
					find_candidates(B.P, B.P, c.nbh_h);
					find_candidates(B.Q, B.P, c.nbh_h);
				}
			}
		}
		if (c.method != UL && c.method != UL_WEAK) recorded = true;
	}

	// tensile.cpp:776-807: element map, 2x2 Gauss points, neighbours, RKPM
	void setup_weak(Body& B, const BodyIn& in);
};

// element_map_rectangle, element.cpp:23-39
std::vector<Elem> element_map_rectangle(unsigned ex, unsigned ey) {
	std::vector<Elem> map;
	unsigned nx = ex + 1;
	const unsigned pattern[4] = {0, 1, nx + 1, nx};
	unsigned inc = 0;
	for (unsigned i = 0; i < ey; i++) {
		for (unsigned j = 0; j < ex; j++) {
			map.push_back(Elem{pattern[0] + inc, pattern[1] + inc, pattern[2] + inc, pattern[3] + inc});
			inc++;
		}
		inc = (i + 1) * nx;
	}
	return map;
}

// gauss_int::update_gauss_points (gauss_integration.h:47-123): per element the Gauss
// points of the tensor rule of `order` (gauss_integration.cpp:20-34 shape functions,
// :38-64 abscissae, :127-141 tensor rule) placed by the nodes' positions (nx, ny):
// the points' x = X, their weights J w, and as their neighbours the element's nodes in
// node order with the element's shape functions and gradients.
void update_gauss_points(PSet& Q, const std::vector<double>& nx, const std::vector<double>& ny,
                         const std::vector<Elem>& elems, unsigned order) {
	double p1[2], w1[2];
	if (order == 1) { p1[0] = 0.; w1[0] = 2.; }
	else if (order == 2) { p1[0] = 0.577350269189626; p1[1] = -0.577350269189626; w1[0] = w1[1] = 1.000000000000000; }
	else throw Fail{"gauss: orders 1 and 2 only"};
	const unsigned npe = order * order;
	double lx[4], ly[4], lw[4];
	for (unsigned i = 0, k = 0; i < order; i++)
		for (unsigned j = 0; j < order; j++, k++) { lx[k] = p1[i]; ly[k] = p1[j]; lw[k] = w1[i] * w1[j]; }
	unsigned g = 0;
	for (const Elem& e : elems) {
		unsigned node_idx[4] = {e.ll, e.lr, e.tr, e.tl};
		glm::dmat2x4 m_node, m_node_par;
		for (int I = 0; I < 4; I++) { m_node[0][I] = nx[node_idx[I]]; m_node[1][I] = ny[node_idx[I]]; }
		m_node_par[0][0] = -1; m_node_par[1][0] = -1;
		m_node_par[0][1] = +1; m_node_par[1][1] = -1;
		m_node_par[0][2] = +1; m_node_par[1][2] = +1;
		m_node_par[0][3] = -1; m_node_par[1][3] = +1;
		for (unsigned i = 0; i < npe; i++) {
			double xi = lx[i], eta = ly[i], local_w = lw[i];
			const double X1 = -1, Y1 = -1, X2 = 1, Y2 = -1, X3 = 1, Y3 = 1, X4 = -1, Y4 = 1;
			glm::dvec4 N;
			glm::dmat2x4 N_xi;
			N[0] = 0.25 * (1 + X1 * xi) * (1 + Y1 * eta);
			N[1] = 0.25 * (1 + X2 * xi) * (1 + Y2 * eta);
			N[2] = 0.25 * (1 + X3 * xi) * (1 + Y3 * eta);
			N[3] = 0.25 * (1 + X4 * xi) * (1 + Y4 * eta);
			N_xi[0][0] = 0.25 * X1 * (1 + Y1 * eta); N_xi[1][0] = 0.25 * Y1 * (1 + X1 * xi);
			N_xi[0][1] = 0.25 * X2 * (1 + Y2 * eta); N_xi[1][1] = 0.25 * Y2 * (1 + X2 * xi);
			N_xi[0][2] = 0.25 * X3 * (1 + Y3 * eta); N_xi[1][2] = 0.25 * Y3 * (1 + X3 * xi);
			N_xi[0][3] = 0.25 * X4 * (1 + Y4 * eta); N_xi[1][3] = 0.25 * Y4 * (1 + X4 * xi);
			glm::dvec2 gpos = glm::transpose(m_node) * N;
			Q.x[g] = gpos[0]; Q.y[g] = gpos[1];
			Q.X[g] = gpos[0]; Q.Y[g] = gpos[1];
			glm::dmat2x2 x_xi(0.);
			for (unsigned I = 0; I < 4; I++) {
				double x_xi11 = 0.25 * m_node[0][I] * m_node_par[0][I] * (1 + m_node_par[1][I] * eta);
				double x_xi12 = 0.25 * m_node[0][I] * m_node_par[1][I] * (1 + m_node_par[0][I] * xi);
				double x_xi21 = 0.25 * m_node[1][I] * m_node_par[0][I] * (1 + m_node_par[1][I] * eta);
				double x_xi22 = 0.25 * m_node[1][I] * m_node_par[1][I] * (1 + m_node_par[0][I] * xi);
				x_xi += glm::dmat2x2(x_xi11, x_xi21, x_xi12, x_xi22);
			}
			double J = -glm::determinant(x_xi);
			double wgt = local_w * J;
			if (!(wgt > 0.)) throw Fail{"gauss: non-positive weight (gauss_integration.h:103)"};
			Q.qw[g] = wgt;
			glm::dmat2x2 x_xi_inv = glm::inverse(x_xi);
			glm::dmat2x4 N_x = N_xi * x_xi_inv;
			Q.num_nbh[g] = 4;
			for (unsigned I = 0; I < 4; I++) {
				size_t o = (size_t)g * MAX_NBH + I;
				Q.nbh[o] = node_idx[I];
				Q.w[o] = N[I];
				Q.w_x[o] = N_x[0][I];
				Q.w_y[o] = N_x[1][I];
			}
			g++;
		}
	}
}

// Weak TL set-up: update_gauss_points on the element map, their weights J w and the
// elements' own shape functions.  The element geometry is the particles' reference position X: the
// set-ups call it before they move any body.  With an explicit element map the Gauss
// points' x, y, h and rho come from the case (as the set-up left them, e.g. shifted
// with their body); otherwise x = X, h = gp_h, rho = gp_rho.  SHAPE_RKPM then replaces
// the element functions by neighbour search + RKPM (tensile.cpp:797-801, rings.cpp:1015-1025);
// SHAPE_ELEMENT keeps them (the *_fem set-ups) and gives the particles no lists.
void Sim::setup_weak(Body& B, const BodyIn& in) {
	std::vector<Elem> elems;
	if (in.ex) {
		elems = element_map_rectangle(in.ex, in.ey);
	} else {
		for (size_t e = 0; e + 3 < in.quads.size(); e += 4)
			elems.push_back(Elem{in.quads[e], in.quads[e + 1], in.quads[e + 2], in.quads[e + 3]});
	}
	const unsigned order = in.ex ? 2 : in.order;
	unsigned ngp = order * order * (unsigned)elems.size();
	B.Q.resize(ngp);
	for (int s = 0; s < 4; s++) B.kq[s].resize(ngp);
	PSet& Q = B.Q;
	update_gauss_points(Q, B.P.X, B.P.Y, elems, order);
	const bool given = !in.ex && in.ngp == ngp;
	for (unsigned i = 0; i < ngp; i++) {
		Q.h[i] = given ? in.g[6][i] : c.gp_h;
		Q.rho[i] = given ? in.g[5][i] : c.gp_rho;
		if (given) { Q.x[i] = in.g[0][i]; Q.y[i] = in.g[1][i]; }
	}
	if (!in.ex && in.shape == SHAPE_ELEMENT) return;
	find_neighbors(B.P, B.P, c.nbh_h, c.nbh_eps);
	find_neighbors(Q, B.P, c.nbh_h, c.nbh_eps);
	precomp_rkpm(Q, B.P);
	precomp_rkpm(B.P, B.P);
}

}  // namespace

int main(int argc, char** argv) {
	if (argc < 3) {
		fprintf(stderr, "usage: %s CASE RESULT\n", argv[0]);
		return 2;
	}
	Sim sim;
	sim.c = read_case(argv[1]);
	Writer w(argv[2]);
	w.raw("MFOUT1\0\0", 8);
	w.u32(sim.c.nbodies);
	for (auto& b : sim.c.bodies) w.u32(b.n);
	try {
		sim.setup();
		auto dump = [&](unsigned step) {
			w.u32(1);
			w.u32(step);
			w.f64(sim.ctx.time);
			for (auto& B : sim.bodies) {
				const std::vector<double>* a[NOUT] = {&B.P.x, &B.P.y, &B.P.vx, &B.P.vy, &B.P.rho, &B.P.Sxx, &B.P.Sxy, &B.P.Syy, &B.P.fcx, &B.P.fcy};
				for (int k = 0; k < NOUT; k++) w.raw(a[k]->data(), B.n * 8);
			}
		};
		double secs = 0.;
		unsigned warm = argc > 3 ? (unsigned)atoi(argv[3]) : 0u;  // steps excluded from the timing
		for (unsigned s = 1; s <= sim.c.nsteps; s++) {
			auto t0 = std::chrono::steady_clock::now();
			sim.driver_step();
			if (s > warm) secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
			if ((sim.c.dump_every && s % sim.c.dump_every == 0) || s == sim.c.nsteps) dump(s);
		}
		if (sim.c.nsteps == 0) dump(0);
		w.u32(2);
		for (unsigned b = 0; b < sim.bodies.size(); b++) {
			auto& L = sim.first_nbh[b];
			unsigned n = sim.bodies[b].n;
			w.u32(n);
			for (unsigned i = 0; i < n; i++) w.u32(i < L.size() ? (uint32_t)L[i].size() : 0u);
			for (unsigned i = 0; i < n && i < L.size(); i++) w.raw(L[i].data(), L[i].size() * 4);
		}
		w.u32(3);
		w.f64(secs);
		w.u32(0);
	} catch (Fail& f) {
		w.u32(9);
		fprintf(stderr, "oracle error: %s\n", f.what);
		return 3;
	}
	return 0;
}
