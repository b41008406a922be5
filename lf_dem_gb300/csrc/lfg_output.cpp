// lfg_output.cpp -- LF_DEM's text output files for a simulation advanced by
// the engine, column for column:
//  - data_<name>.dat : Simulation::outputData (Simulation.cpp:641-780)
//  - st_<name>.dat   : its stress-tensor part (Simulation.cpp:781-792)
//  - par_<name>.dat  : Simulation::outputParFileTxt (Simulation.cpp:884-965)
//  - int_<name>.dat  : Simulation::outputIntFileTxt (Simulation.cpp:967-1006)
//  - pst_<name>.dat  : Simulation::outputPstFileTxt (Simulation.cpp:823-852),
//                      when out_particle_stress names groups
// each file starting with Simulation::createDataHeader (Simulation.cpp:
// 857-869), the per-snapshot blocks of par_/int_ with getSnapshotHeader
// (Simulation.cpp:811-836).  The column mechanics follow OutputData
// (OutputData.h:27-209): a value is multiplied by the converter of its
// physical dimension (the internal-to-output force ratio) and printed by an
// ostream with the column's precision; the first write puts "# data in
// <unit> units." and one "#i: name" / "#i-j: name" line per column.
// Scope: simple shear, no walls, no Brownian or cohesive forces (what the
// engine runs).  int_ rows are sorted by particle pair (the reference writes
// its interaction vector's order, which depends on creation history).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "lfg_internal.h"
#include "lfg_physics.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);
int ok(lfg_status *st);
int sim_output_snapshot(lfg_sim *h, OutputSnapshot &o);
}
using lfg::fail;
using lfg::ok;

namespace {

// One output file in OutputData's format.
class Table {
public:
	bool open(const std::string &path, const std::string &file_header, bool overwrite)
	{
		if (!overwrite) {
			std::ifstream probe(path.c_str());
			if (probe.good()) return false;
		}
		out_.open(path.c_str(), std::ofstream::out);
		if (!out_.good()) return false;
		out_ << file_header;
		return true;
	}
	// OutputData::setDimensionlessNumber (OutputData.h:112-125)
	void set_units(const std::string &unit, double d)
	{
		unit_ = unit;
		if (d == 0) d = 1;
		conv_ = {{"none", 1}, {"viscosity", 6*M_PI}, {"stress", 6*M_PI*d}, {"force", d},
		         {"time", 1/d}, {"rate", d}, {"velocity", d}};
	}
	void set_precision(int p) { precision_ = p; }
	// OutputData::entryData: width values printed as one column group
	void entry(const std::string &name, const std::string &dim, int width, const double *v, int precision = -1)
	{
		auto it = index_.find(name);
		if (it == index_.end()) {
			index_[name] = (int)cols_.size();
			cols_.push_back(Col{name, dim, width, {}});
			it = index_.find(name);
		}
		Col &c = cols_[it->second];
		double k = conv_[c.dim];
		std::ostringstream s;
		s << std::setprecision(precision > 0 ? precision : precision_);
		for (int e = 0; e < width; e++) {   // vec3d / Sym2Tensor print their elements space-separated
			if (e) s << ' ';
			s << k*v[e];
		}
		c.rows.push_back(s.str());
	}
	void entry1(const std::string &name, const std::string &dim, double v, int precision = -1)
	{
		entry(name, dim, 1, &v, precision);
	}
	// OutputData::writeToFile (OutputData.h:160-209)
	void write(const std::string &block_header)
	{
		if (first_) {
			out_ << "# data in " << unit_ << " units." << std::endl;
			int i = 1;
			for (const Col &c : cols_) {
				if (c.width == 1) out_ << "#" << i << ": ";
				else out_ << "#" << i << "-" << i+c.width-1 << ": ";
				i += c.width;
				out_ << c.name << std::endl;
			}
			out_ << std::endl;
			first_ = false;
		}
		out_ << block_header;
		size_t lines = 0;
		for (const Col &c : cols_) if (!c.rows.empty()) { lines = c.rows.size(); break; }
		for (size_t r = 0; r < lines; r++) {
			for (const Col &c : cols_) out_ << (c.rows.empty() ? std::string("n") : c.rows[r]) << " ";
			out_ << std::endl;
		}
		for (Col &c : cols_) c.rows.clear();
		out_.flush();
	}
	bool good() const { return out_.good(); }

private:
	struct Col {
		std::string name, dim;
		int width;
		std::vector<std::string> rows;
	};
	std::ofstream out_;
	std::string unit_;
	std::map<std::string, double> conv_;
	std::map<std::string, int> index_;
	std::vector<Col> cols_;
	int precision_ = 6;
	bool first_ = true;
};

double ddot(const double *a, const double *b)   // doubledot (Sym2Tensor.h:246-254)
{
	return a[0]*b[0]+2*a[1]*b[1]+2*a[2]*b[2]+2*a[3]*b[3]+a[4]*b[4]+a[5]*b[5];
}
double selfddot(const double *a)   // Sym2Tensor::selfdoubledot (Sym2Tensor.h:114-122)
{
	return a[0]*a[0]+2*a[1]*a[1]+2*a[2]*a[2]+2*a[3]*a[3]+a[4]*a[4]+a[5]*a[5];
}
double vnorm(const double *v) { return std::sqrt(v[0]*v[0]+v[1]*v[1]+v[2]*v[2]); }
double vdot3(const double *a, const double *b) { return a[0]*b[0]+a[1]*b[1]+a[2]*b[2]; }

} // namespace

struct lfg_output {
	lfg_sim *sim = nullptr;
	lfg_output_config cfg;
	std::string unit, version, pst_letters;
	Table data, st, par, inter, pst;
	int flags = 0;   // 1 par_, 2 int_
};

namespace {

// Simulation::getSnapshotHeader (Simulation.cpp:811-836), simple shear
std::string snapshot_header(const lfg_output &o, const lfg::OutputSnapshot &S)
{
	std::stringstream h;
	const std::string sep = " : ";
	h << "# cumulated strain" << sep << S.strain << std::endl;
	h << "# shear disp" << sep << S.shear_disp[0] << std::endl;
	// Simulation::getRate: the input rate (rate control), the internal
	// shear rate (stress control)
	h << "# shear rate" << sep << (S.control == 0 ? o.cfg.input_value : S.shear_rate) << std::endl;
	if (S.control == 1) h << "# target stress" << sep << o.cfg.input_value << std::endl;
	return h.str();
}

void write_data(lfg_output &o, const lfg::OutputSnapshot &S)
{
	Table &T = o.data;
	const double sr = S.shear_rate;
	// Einf_base and the stress bases of simple shear (SimulationInit.cpp:650-662)
	const double d = 0.5;
	const double Eb[6] = {0, 0, d, 0, 0, 0};
	const double B0[6] = {-d/2, 0, 0, 0, d, -d/2}, B3[6] = {-d, 0, 0, 0, 0, d};
	const double *sig = S.total_stress;
	double viscosity, inv0, inv3;
	if (sr != 0) {
		viscosity = 0.5*ddot(sig, S.Einf)/selfddot(S.Einf);
		inv0 = ddot(sig, B0)/selfddot(B0);
		inv3 = ddot(sig, B3)/selfddot(B3);
	} else {
		viscosity = 0.5*ddot(sig, Eb)/selfddot(Eb);
		inv0 = 0;
		inv3 = 0;
	}
	T.entry1("time", "time", S.time);
	T.entry1("cumulated shear strain", "none", S.strain);
	T.entry1("shear rate", "rate", S.shear_rate);
	T.entry1("viscosity", "viscosity", viscosity);
	for (size_t g = 0; g < S.groups.size(); g++) {
		double c = ddot(S.group_stress[g].data(), S.Einf)/selfddot(S.Einf);
		T.entry1("Viscosity("+S.groups[g]+")", "viscosity", 0.5*c);
	}
	T.entry1("inviscid function 0th", "viscosity", inv0);
	T.entry1("inviscid function 3rd", "viscosity", inv3);
	T.entry1("N1 viscosity", "viscosity", (sig[0]-sig[5])/sr);
	T.entry1("N2 viscosity", "viscosity", (sig[5]-sig[4])/sr);
	T.entry1("particle pressure", "stress", -(sig[0]+sig[4]+sig[5])/3);
	double pc = 0;
	for (size_t g = 0; g < S.groups.size(); g++)
		if (S.groups[g] == "contact") {
			const double *c = S.group_stress[g].data();
			pc = -(c[0]+c[4]+c[5])/3;
		}
	T.entry1("particle pressure contact", "stress", pc);
	// SystemHelperFunctions.h: getPotentialEnergy, evaluateMinGap,
	// evaluateMaxDispTan, evaluateMaxDispRolling, countNumberOfContact
	const int W = S.out_w;
	const size_t npair = S.pairs.size()/W;
	double energy = 0, min_gap = S.interaction_range, max_dt = 0, max_dr = 0;
	unsigned contacts = 0, frictional = 0;
	for (size_t t = 0; t < npair; t++) {
		const double *r = S.pairs.data()+t*W;
		bool contact = ((int)r[0] & lfg::PF_CONTACT) != 0;
		if (contact) energy += r[21];
		if (S.repulsion) energy += r[22];
		if (r[4] < min_gap) min_gap = r[4];
		max_dt = std::max(max_dt, vnorm(r+23));
		max_dr = std::max(max_dr, vnorm(r+26));
		if (contact) {
			contacts++;
			if ((int)r[3] >= 2) frictional++;
		}
	}
	T.entry1("energy", "none", energy);
	T.entry1("min gap", "none", min_gap);
	T.entry1("max tangential displacement", "none", max_dt);
	T.entry1("max rolling displacement", "none", max_dr);
	T.entry1("contact number", "none", (double)2*contacts/S.n);
	T.entry1("frictional contact number", "none", (double)2*frictional/S.n);
	T.entry1("number of interaction", "none", (double)npair);
	T.entry1("max velocity", "velocity", S.max_velocity);
	double max_w = 0;   // evaluateMaxAngVelocity (SystemHelperFunctions.h:4-14)
	for (int i = 0; i < S.n; i++) max_w = std::max(max_w, vnorm(S.na.data()+6*i+3));
	T.entry1("max angular velocity", "velocity", max_w);
	T.entry1("dt", "time", S.avg_dt);
	T.entry1("kn", "none", S.kn);
	T.entry1("kt", "none", S.kt);
	T.entry1("kr", "none", S.kr);
	T.entry("shear strain", "none", 3, S.shear_strain);
	T.write("");
	Table &U = o.st;
	U.entry1("time", "time", S.time);
	U.entry1("cumulated strain", "none", S.strain);
	U.entry1("shear rate", "rate", S.shear_rate);
	U.entry("total stress tensor (xx, xy, xz, yz, yy, zz)", "stress", 6, S.total_stress);
	for (size_t g = 0; g < S.groups.size(); g++)
		U.entry(S.groups[g]+" stress tensor (xx, xy, xz, yz, yy, zz)", "stress", 6, S.group_stress[g].data());
	U.write("");
}

void write_par(lfg_output &o, const lfg::OutputSnapshot &S)
{
	Table &T = o.par;
	const int n = S.n;
	const double lx = S.lx, ly = S.ly, lz = S.lz;
	for (int i = 0; i < n; i++) {
		double p[3] = {S.pos[3*i], S.pos[3*i+1], S.pos[3*i+2]};
		double v[3] = {S.vel[3*i], S.vel[3*i+1], S.vel[3*i+2]};
		if (o.cfg.origin_zero_flow) {
			// Simulation::shiftUpCoordinate (Simulation.cpp:838-855)
			double x = p[0]-0.5*lx, y = p[1]-0.5*ly, z = p[2]-0.5*lz;
			z += 0.5*lz;
			if (z > 0.5*lz) {
				x -= S.shear_disp[0];
				y -= S.shear_disp[1];
				if (x < -0.5*lx) x += lx;
				if (y < -0.5*ly) y += ly;
				z -= lz;
			}
			p[0] = x; p[1] = y; p[2] = z;
			if (p[2] < 0)
				for (int k = 0; k < 3; k++) v[k] -= S.vel_diff[k];
		}
		T.entry1("particle index", "none", (double)i);
		T.entry1("radius", "none", S.radius[i]);
		T.entry("position (x, y, z)", "none", 3, p, 6);
		T.entry("velocity (x, y, z)", "velocity", 3, v);
		T.entry("angular velocity (x, y, z)", "none", 3, S.ang.data()+3*i);
		T.entry("non affine displacement (x, y, z)", "none", 3, S.na_disp.data()+3*i);
		if (S.twodim) T.entry1("angle", "none", S.angle[i]);
	}
	T.write(snapshot_header(o, S));
}

void write_int(lfg_output &o, const lfg::OutputSnapshot &S)
{
	Table &T = o.inter;
	const int W = S.out_w;
	const size_t npair = S.pairs.size()/W;
	const bool full = !o.cfg.diminish_output;
	const double sr = S.shear_rate;
	double Esr[6];
	for (int e = 0; e < 6; e++) Esr[e] = S.Einf[e]/sr;
	for (size_t t = 0; t < npair; t++) {
		const double *r = S.pairs.data()+t*W;
		const double *nv = r+5;
		T.entry1("particle 1 label", "none", r[1]);
		T.entry1("particle 2 label", "none", r[2]);
		T.entry1("contact state (0 = no contact, 1 = frictionless contact, 2 = non-sliding frictional, "
		         "3 = sliding frictional)", "none", r[3]);
		if (full) {
			T.entry("normal vector, oriented from particle 1 to particle 2", "none", 3, nv);
			T.entry1("dimensionless gap = s-2, s = 2r/(a1+a2)", "none", r[4]);
		}
		if (S.lubrication) {
			double fn = 0, ft[3] = {0, 0, 0};
			if (r[4] > 0) {
				const double *f = r+8;
				fn = -vdot3(f, nv);
				double c = vdot3(f, nv);
				for (int k = 0; k < 3; k++) ft[k] = f[k]-c*nv[k];
			}
			T.entry1("normal part of the lubrication force (positive for compression)", "force", fn);
			T.entry("tangential part of the lubrication force", "force", 3, ft);
		}
		const double *F = r+11;
		double c = vdot3(nv, F), Fn[3], Ft[3];
		for (int k = 0; k < 3; k++) { Fn[k] = c*nv[k]; Ft[k] = F[k]-c*nv[k]; }
		T.entry1("norm of the normal part of the contact force", "force", vnorm(Fn));
		T.entry("tangential part of the contact force", "force", 3, Ft);
		T.entry1("norm of the normal repulsive force", "force", r[14]);
		if (full) T.entry1("Viscosity contribution of contact xF", "stress", ddot(r+15, Esr)/sr);
	}
	if (npair > 0) T.write(snapshot_header(o, S));
}

// The stress components System::declareStressComponents (Stress.cpp:20-75)
// creates, in the key order of its std::map (which fixes the order of the
// per-particle sums), with the engine's slot and the component's group.
struct PstComponent { const char *key; int slot; const char *group; };
const PstComponent PST_COMPONENTS[] = {
	{"M_E_hydro", lfg::SC_ME, "hydro"},
	{"brownian", lfg::SC_GU_BROWNIAN, "brownian"},
	{"brownian_predictor", lfg::SC_BROWNIAN_PRED, "brownian"},
	{"contact", lfg::SC_GU_CONTACT, "contact"},
	{"dashpot", lfg::SC_GU_DASHPOT, "dashpot"},
	{"hydro", lfg::SC_GU_HYDRO, "hydro"},
	{"repulsion", lfg::SC_GU_REPULSION, "repulsion"},
	{"xF_contact", lfg::SC_XF_CONTACT, "contact"},
	{"xF_contact_rateindep", lfg::SC_XF_RATEINDEP, "contact"},
	{"xF_contact_rateprop", lfg::SC_XF_RATEPROP, "contact"},
	{"xF_repulsion", lfg::SC_XF_REPULSION, "repulsion"},
};

// Simulation::outputPstFileTxt (Simulation.cpp:823-852): the groups the
// letters name (Simulation.cpp:832-838; a letter outside the table names the
// empty group) in the order of their names (a std::map), per particle the
// sum of the group's declared components' stresslets in key order
// (Simulation::getParticleStressGroup, Simulation.cpp:628-639; "total": all),
// in stress units.
void write_pst(lfg_output &o, const lfg::OutputSnapshot &S)
{
	static const std::map<char, std::string> shorts = {{'l', "hydro"}, {'c', "contact"}, {'r', "repulsion"},
	                                                   {'b', "brownian"}, {'d', "dashpot"}, {'t', "total"}};
	std::map<std::string, std::vector<int>> groups;   // group -> slots summed, in key order
	for (char ch : o.pst_letters) {
		auto it = shorts.find(ch);
		const std::string g = it == shorts.end() ? std::string() : it->second;
		std::vector<int> &slots = groups[g];
		slots.clear();
		for (const PstComponent &c : PST_COMPONENTS)
			if (S.slot_declared[c.slot] && (g == "total" || g == c.group)) slots.push_back(c.slot);
	}
	Table &T = o.pst;
	const int n = S.n;
	for (int i = 0; i < n; i++)
		for (const auto &g : groups) {
			double v[6] = {0, 0, 0, 0, 0, 0};
			for (int slot : g.second) {
				const double *x = S.particle_stress.data()+((size_t)slot*n+i)*6;
				for (int e = 0; e < 6; e++) v[e] += x[e];
			}
			T.entry(g.first+" stress (xx, xy, xz, yz, yy, zz)", "stress", 6, v);
		}
	T.write(snapshot_header(o, S));
}

} // namespace

extern "C" {

int lfg_output_open(lfg_sim *sim, const lfg_output_config *cfg, lfg_output **out, lfg_status *st)
{
	if (!sim || !cfg || !out || !cfg->simu_name || !cfg->unit) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	lfg::OutputSnapshot S;
	try {
		lfg::sim_output_snapshot(sim, S);
	} catch (const lfg::Error &e) {
		return fail(st, e.code, e.info, e.msg.c_str());
	}
	lfg_output *o = new lfg_output;
	o->sim = sim;
	o->cfg = *cfg;
	o->unit = cfg->unit;
	o->version = cfg->version ? cfg->version : "lf_dem_gb300";
	o->cfg.unit = o->unit.c_str();
	o->cfg.version = o->version.c_str();
	// Simulation::createDataHeader (Simulation.cpp:857-869)
	std::stringstream h;
	h << "# LF_DEM version " << o->version << std::endl;
	h << "# np " << S.n << std::endl;
	h << "# VF " << cfg->volume_fraction << std::endl;
	h << "# Lx " << S.lx << std::endl;
	h << "# Ly " << S.ly << std::endl;
	h << "# Lz " << S.lz << std::endl;
	h << "# flow_type " << "shear" << std::endl;
	std::string dir = cfg->directory && cfg->directory[0] ? std::string(cfg->directory)+"/" : std::string();
	std::string name = cfg->simu_name;
	bool ow = cfg->force_overwrite != 0;
	bool good = o->data.open(dir+"data_"+name+".dat", h.str(), ow) && o->st.open(dir+"st_"+name+".dat", h.str(), ow);
	if (good && cfg->out_data_particle) good = o->par.open(dir+"par_"+name+".dat", h.str(), ow);
	if (good && cfg->out_data_interaction) good = o->inter.open(dir+"int_"+name+".dat", h.str(), ow);
	o->pst_letters = cfg->out_particle_stress ? cfg->out_particle_stress : "";
	o->cfg.out_particle_stress = o->pst_letters.c_str();
	if (good && !o->pst_letters.empty()) good = o->pst.open(dir+"pst_"+name+".dat", h.str(), ow);
	if (!good) {
		delete o;
		return fail(st, LFG_ERR_BAD_ARG, 0, "cannot create the output files (existing files need force_overwrite)");
	}
	const double d = cfg->internal_to_output;
	for (Table *t : {&o->data, &o->st, &o->par, &o->inter, &o->pst}) t->set_units(o->unit, d);
	// Simulation::outputParFileTxt: precision 4 with diminish_output
	o->par.set_precision(cfg->diminish_output ? 4 : 6);
	o->inter.set_precision(cfg->diminish_output ? 4 : 6);
	*out = o;
	return ok(st);
}

int lfg_output_write(lfg_output *o, lfg_status *st)
{
	if (!o) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	try {
		lfg::OutputSnapshot S;
		S.want_particle_stress = !o->pst_letters.empty();
		lfg::sim_output_snapshot(o->sim, S);
		write_data(*o, S);
		if (o->cfg.out_data_particle) write_par(*o, S);
		if (o->cfg.out_data_interaction) write_int(*o, S);
		if (!o->pst_letters.empty()) write_pst(*o, S);
	} catch (const lfg::Error &e) {
		return fail(st, e.code, e.info, e.msg.c_str());
	}
	if (!o->data.good() || !o->st.good()) return fail(st, LFG_ERR_BAD_ARG, 0, "write error");
	return ok(st);
}

void lfg_output_close(lfg_output *o) { delete o; }

} // extern "C"
