// lfg_config.cpp -- LF_DEM's Parameter_File reader and unit system, so the
// engine runs from the same inputs as the reference CLI (`LF_DEM -r 1r conf
// params` / `-s 10cl`).  Restates SimulationInit.cpp: setDefaultParameters
// (:945-1010), autoSetParameters (:745-889), readParameterFile (:891-943),
// tagStrainParameters (:497-522), setupNonDimensionalization* (:250-346,
// 448-471), resolveUnitSystem (:156-225), catchForcesInStressUnits
// (:227-240), changeUnit (:348-367), exportForceAmplitudes (:396-446),
// assertParameterCompatibility (:473-495) and resolveTimeOrStrainParameters
// (:524-566), then the parameter rewrites of System::setupParameters
// (System.cpp:348-414).  Values are resolved exactly as the reference does:
// the same maps (iterated in key order), the same products and quotients.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>

#include "lfg_internal.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);
int ok(lfg_status *st);
}

namespace {

struct DimVal {
	std::string type;   // "force" or "time"
	double *value = nullptr;
	std::string unit;
};

struct Params {
	int simulation_mode = 0, friction_model = 1, integration_method = 1, np_fixed = 0;
	int nb_output_data_log_time = 0, nb_output_config_log_time = 0;
	bool monolayer = false, log_time_interval = false, out_data_particle = true, out_data_interaction = true;
	bool out_data_vel_components = false, origin_zero_flow = true, auto_determine_knkt = false, fixed_dt = false;
	bool out_bond_order_parameter6 = false, out_binary_conf = false, keep_input_strain = false;
	std::string lubrication_model, event_handler, out_particle_stress;
	double repulsion = 0, cohesion = 0, brownian = 0, critical_load = 0, ft_max = 0;
	double repulsive_length = 0, repulsive_max_length = 0, vdW_coeffient = 0, vdW_singularity_cutoff = 0;
	double lub_reduce_parameter = 0, contact_relaxation_time = 0, contact_relaxation_time_tan = 0;
	double disp_max = 0, dt_max = 0, dt_min = 0, time_end = 0, lub_max_gap = 0, interaction_range = 0;
	double sd_coeff = 0, kn = 0, kt = 0, kr = 0, dt = 0, Pe_switch = 0;
	double mu_static = 0, mu_dynamic = 0, mu_rolling = 0;
	double time_interval_output_config = 0, time_interval_output_data = 0, initial_log_time = 0;
	double overlap_target = 0, disp_tan_target = 0, memory_strain_avg = 0, memory_strain_k = 0, start_adjust = 0;
	double min_kn_auto_det = 0, max_kn_auto_det = 0, min_kt_auto_det = 0, max_kt_auto_det = 0;
	double min_dt_auto_det = 0, max_dt_auto_det = 0, rest_threshold = 0, theta_shear = 0, strain_reversal = 0;
	double brownian_relaxation_time = 0;
};

bool str2bool(const std::string &v)
{
	if (v == "true") return true;
	if (v == "false") return false;
	throw std::runtime_error("the value should be true or false");
}

// the first letter other than 'e' starts the unit suffix (global.h:72-82)
bool get_suffix(const std::string &s, std::string &num, std::string &suf)
{
	size_t p = s.find_first_of("abcdfghijklmnopqrstuvwxyz");
	num = s.substr(0, p);
	if (p == std::string::npos) return false;
	suf = s.substr(p);
	return true;
}

class Resolver {
public:
	Params p;
	double dimensionless_rate = 0;
	double target_stress = 0, shear_rate = 0;
	bool repulsiveforce = false, critical_load_on = false;
	std::map<std::string, DimVal> input_values;
	std::map<std::string, double> force_ratios;
	std::map<std::string, std::string> longname;
	std::map<std::string, double *> force_ptr;

	Resolver()
	{
		longname = {{"h", "hydro"}, {"r", "repulsion"}, {"b", "brownian"}, {"c", "cohesion"},
		            {"cl", "critical_load"}, {"ft", "ft_max"}, {"kn", "kn"}, {"kt", "kt"}, {"kr", "kr"},
		            {"s", "stress"}};
		force_ptr = {{"hydro", &dimensionless_rate}, {"repulsion", &p.repulsion},
		             {"critical_load", &p.critical_load}, {"cohesion", &p.cohesion}, {"ft_max", &p.ft_max},
		             {"brownian", &p.brownian}, {"kn", &p.kn}, {"kt", &p.kt}, {"kr", &p.kr}};
	}

	DimVal dimval(const std::string &type, const std::string &name, const std::string &value, double *ptr)
	{
		std::string num, suf;
		if (!get_suffix(value, num, suf))
			throw std::runtime_error("no unit scale (suffix) provided for "+name);
		auto it = longname.find(suf);
		DimVal v;
		v.type = type;
		v.value = ptr;
		v.unit = it == longname.end() ? std::string() : it->second;
		*ptr = std::atof(num.c_str());
		return v;
	}

	void force(const std::string &k, const std::string &v) { input_values[k] = dimval("force", k, v, force_ptr.at(k)); }
	void time(const std::string &k, const std::string &v, double *ptr) { input_values[k] = dimval("time", k, v, ptr); }
	void forcep(const std::string &k, const std::string &v, double *ptr) { input_values[k] = dimval("force", k, v, ptr); }

	// SimulationInit.cpp:745-889
	void set(const std::string &k, const std::string &v)
	{
		auto f = [&](const char *n) { return k == n; };
		double a = std::atof(v.c_str());
		int i = std::atoi(v.c_str());
		if (f("simulation_mode")) p.simulation_mode = i;
		else if (f("lubrication_model")) p.lubrication_model = v;
		else if (f("friction_model")) p.friction_model = i;
		else if (f("repulsion") || f("cohesion") || f("brownian") || f("critical_load") || f("kn") || f("kt") ||
		         f("kr") || f("ft_max")) force(k, v);
		else if (f("monolayer")) p.monolayer = str2bool(v);
		else if (f("repulsive_length")) p.repulsive_length = a;
		else if (f("repulsive_max_length")) p.repulsive_max_length = a;
		else if (f("vdW_coeffient")) p.vdW_coeffient = a;
		else if (f("vdW_singularity_cutoff")) p.vdW_singularity_cutoff = a;
		else if (f("lub_reduce_parameter")) p.lub_reduce_parameter = a;
		else if (f("contact_relaxation_time")) time(k, v, &p.contact_relaxation_time);
		else if (f("contact_relaxation_time_tan")) time(k, v, &p.contact_relaxation_time_tan);
		else if (f("disp_max")) p.disp_max = a;
		else if (f("dt_max")) p.dt_max = a;
		else if (f("dt_min")) p.dt_min = a;
		else if (f("time_end")) time(k, v, &p.time_end);
		else if (f("integration_method")) p.integration_method = i;
		else if (f("lub_max_gap")) p.lub_max_gap = a;
		else if (f("interaction_range")) p.interaction_range = a;
		else if (f("sd_coeff")) p.sd_coeff = a;
		else if (f("dt")) p.dt = a;
		else if (f("Pe_switch")) p.Pe_switch = a;
		else if (f("mu_static")) p.mu_static = a;
		else if (f("mu_dynamic")) p.mu_dynamic = a;
		else if (f("mu_rolling")) p.mu_rolling = a;
		else if (f("time_interval_output_config")) time(k, v, &p.time_interval_output_config);
		else if (f("time_interval_output_data")) time(k, v, &p.time_interval_output_data);
		else if (f("log_time_interval")) p.log_time_interval = str2bool(v);
		else if (f("initial_log_time")) time(k, v, &p.initial_log_time);
		else if (f("nb_output_data_log_time")) p.nb_output_data_log_time = i;
		else if (f("nb_output_config_log_time")) p.nb_output_config_log_time = i;
		else if (f("out_data_particle")) p.out_data_particle = str2bool(v);
		else if (f("out_data_interaction")) p.out_data_interaction = str2bool(v);
		else if (f("out_data_vel_components")) p.out_data_vel_components = str2bool(v);
		else if (f("origin_zero_flow")) p.origin_zero_flow = str2bool(v);
		else if (f("auto_determine_knkt")) p.auto_determine_knkt = str2bool(v);
		else if (f("overlap_target")) p.overlap_target = a;
		else if (f("disp_tan_target")) p.disp_tan_target = a;
		else if (f("memory_strain_avg")) p.memory_strain_avg = a;
		else if (f("memory_strain_k")) p.memory_strain_k = a;
		else if (f("start_adjust")) p.start_adjust = a;
		else if (f("min_kn_auto_det")) forcep(k, v, &p.min_kn_auto_det);
		else if (f("max_kn_auto_det")) forcep(k, v, &p.max_kn_auto_det);
		else if (f("min_kt_auto_det")) forcep(k, v, &p.min_kt_auto_det);
		else if (f("max_kt_auto_det")) forcep(k, v, &p.max_kt_auto_det);
		else if (f("min_dt_auto_det")) p.min_dt_auto_det = a;
		else if (f("max_dt_auto_det")) p.max_dt_auto_det = a;
		else if (f("rest_threshold")) p.rest_threshold = a;
		else if (f("fixed_dt")) p.fixed_dt = str2bool(v);
		else if (f("theta_shear")) p.theta_shear = a*M_PI/180;
		else if (f("strain_reversal")) p.strain_reversal = a;
		else if (f("event_handler")) p.event_handler = v;
		else if (f("out_particle_stress")) {
			// quotes removed (SimulationInit.cpp:871-873)
			p.out_particle_stress.clear();
			for (char ch : v) if (ch != '"') p.out_particle_stress += ch;
		}
		else if (f("out_bond_order_parameter6")) p.out_bond_order_parameter6 = str2bool(v);
		else if (f("out_binary_conf")) p.out_binary_conf = str2bool(v);
		else if (f("np_fixed")) p.np_fixed = i;
		else if (f("keep_input_strain")) p.keep_input_strain = str2bool(v);
		else if (f("brownian_relaxation_time")) p.brownian_relaxation_time = a;
		else throw std::runtime_error("keyword "+k+" is not associated with a parameter");
	}

	// SimulationInit.cpp:945-1010
	void defaults(const std::string &s)
	{
		set("Pe_switch", "5"); set("dt", "1e-4"); set("disp_max", "1e-3"); set("dt_max", "-1");
		set("monolayer", "false"); set("rest_threshold", "1e-4"); set("integration_method", "1");
		set("np_fixed", "0"); set("sd_coeff", "1"); set("lubrication_model", "tangential");
		set("friction_model", "1"); set("time_end", "10h"); set("lub_max_gap", "0.5");
		set("interaction_range", "-1"); set("lub_reduce_parameter", "1e-3");
		set("contact_relaxation_time", "1e-3"+s); set("contact_relaxation_time_tan", "-1"+s);
		if (s != "kn") { set("kn", "2000"+s); set("min_kn_auto_det", "1000"+s); set("max_kn_auto_det", "1000000"+s); }
		if (s != "kt") { set("kt", "0.5kn"); set("min_kt_auto_det", "1000"+s); set("max_kt_auto_det", "1000000"+s); }
		set("min_dt_auto_det", "1e-7"); set("max_dt_auto_det", "1e-3");
		if (s != "kr") set("kr", "0kn");
		set("auto_determine_knkt", "false"); set("overlap_target", "0.05"); set("disp_tan_target", "0.05");
		set("memory_strain_avg", "0.01"); set("memory_strain_k", "0.02"); set("start_adjust", "0.2");
		set("repulsive_length", "0.05"); set("repulsive_max_length", "-1"); set("vdW_coeffient", "-1");
		set("vdW_singularity_cutoff", "0.1"); set("mu_static", "1"); set("mu_dynamic", "-1");
		set("mu_rolling", "0"); set("time_interval_output_data", "1e-2h"); set("time_interval_output_config", "1e-1h");
		set("log_time_interval", "false"); set("initial_log_time", "1e-4h"); set("nb_output_data_log_time", "100");
		set("nb_output_config_log_time", "100"); set("origin_zero_flow", "true"); set("out_data_particle", "true");
		set("out_data_interaction", "true"); set("out_particle_stress", ""); set("out_binary_conf", "false");
		set("out_data_vel_components", "false"); set("fixed_dt", "false"); set("dt_min", "-1"); set("dt_max", "-1");
		set("theta_shear", "0"); set("event_handler", ""); set("simulation_mode", "0");
		set("keep_input_strain", "false"); set("brownian_relaxation_time", "1"); set("out_bond_order_parameter6", "false");
	}

	// SimulationInit.cpp:891-943: statements end with ';' (text after the
	// last ';' is ignored), all white space is removed, /* */ comments are
	// dropped and // is an error
	void read(const std::string &text)
	{
		size_t pos = 0;
		for (;;) {
			size_t e = text.find(';', pos);
			if (e == std::string::npos) break;
			std::string line = text.substr(pos, e-pos);
			pos = e+1;
			std::string s;
			for (char c : line)
				if (!std::isspace((unsigned char)c)) s += c;
			for (;;) {
				size_t b = s.find("/*");
				if (b == std::string::npos) break;
				size_t c = s.find("*/");
				if (c == std::string::npos || c < b) throw std::runtime_error("syntax error in the parameter file");
				s = s.substr(c+2);
			}
			if (s.find("*/") != std::string::npos) throw std::runtime_error("syntax error in the parameter file");
			if (s.find("//") != std::string::npos)
				throw std::runtime_error("// is not the syntax to comment out; use /* comment */");
			size_t q = s.find('=');
			set(s.substr(0, q), q == std::string::npos ? std::string() : s.substr(q+1));
		}
	}

	void tag_strain()
	{
		for (const char *n : {"time_interval_output_data", "time_interval_output_config", "time_end", "initial_log_time"}) {
			auto &v = input_values[n];
			if (v.unit == "hydro") v.unit = "strain";
		}
	}

	void change_unit(DimVal &x, const std::string &u)
	{
		if (u == x.unit) return;
		if (x.type == "force") {
			*x.value *= force_ratios[x.unit+'/'+u];
			x.unit = u;
		} else if (x.type == "time") {
			if (x.unit != "strain") {
				*x.value /= force_ratios[x.unit+'/'+u];
				x.unit = u;
			}
		} else {
			throw std::runtime_error("no unit change for a value of type "+x.type);
		}
	}

	void resolve(const std::string &uf)
	{
		DimVal inv;
		inv.type = "force";
		inv.value = force_ptr.at(uf);
		inv.unit = uf;
		input_values[uf] = inv;
		*input_values[uf].value = 1;
		for (const auto &x : input_values)
			if (x.second.type == "force") force_ratios[x.first+'/'+x.second.unit] = *x.second.value;
		bool unsolved, solved;
		do {
			unsolved = false;
			solved = false;
			for (auto &x : input_values) {
				const std::string unit = x.second.unit;
				if (unit != uf && unit != "strain") {
					if (force_ratios.find(unit+'/'+uf) != force_ratios.end()) {
						change_unit(x.second, uf);
						if (x.second.type == "force") force_ratios[x.first+'/'+uf] = *x.second.value;
						solved = true;
					} else {
						unsolved = true;
					}
				}
			}
		} while (unsolved && solved);
		if (unsolved) {
			for (const auto &x : input_values)
				if (x.second.unit != uf && x.second.unit != "strain")
					throw std::runtime_error("input value \""+x.first+"\" has an unknown unit \""+x.second.unit+"\"");
		}
		// every pairwise ratio of the resolved forces, both ways, in the same
		// loop order (Simulation::buildFullSetOfForceRatios, SimulationInit.cpp:
		// 136-153): the output converter reads force_ratios[internal/output]
		std::map<std::string, double> forces;
		for (const auto &x : input_values)
			if (x.second.type == "force") forces[x.first] = *x.second.value;
		for (const auto &f1 : forces)
			for (const auto &f2 : forces) {
				force_ratios[f2.first+'/'+f1.first] = f2.second/f1.second;
				force_ratios[f1.first+'/'+f2.first] = 1/force_ratios[f2.first+'/'+f1.first];
			}
	}

	void rate_controlled(double number, const std::string &scale)
	{
		if (input_values.count(scale))
			throw std::runtime_error("redefinition of the rate (given both in the command line and in the parameter file)");
		if (number == 0) throw std::runtime_error("a zero rate (Brownian, rest) is not supported by this engine");
		DimVal inv;
		inv.type = "force";
		inv.value = force_ptr.at(scale);
		inv.unit = "hydro";
		input_values[scale] = inv;
		*input_values[scale].value = 1/number;
		force_ratios[scale+"/hydro"] = *input_values[scale].value;
		resolve("hydro");
		// setUnitScaleRateControlled (SimulationInit.cpp:380-402): with a
		// Brownian force the internal unit stays hydro above Pe_switch; below
		// it the reference switches to Brownian units with time-averaged
		// stresses, which this engine does not run
		if (force_ratios.count("hydro/brownian") || force_ratios.count("brownian/brownian")) {
			if (!(force_ratios["hydro/brownian"] > p.Pe_switch))
				throw std::runtime_error("Brownian-dominated runs (Pe <= Pe_switch) are not supported by this engine");
		}
		for (auto &x : input_values) change_unit(x.second, "hydro");
	}

	void stress_controlled(double number, const std::string &unit)
	{
		if (unit == "hydro") throw std::runtime_error("give a stress in non-hydro units");
		if (unit == "brownian") throw std::runtime_error("Brownian forces are not supported by this engine");
		shear_rate = 0;
		target_stress = number/6/M_PI;
		for (auto &x : input_values) {
			if (x.second.unit == "stress") {
				if (x.second.type != "force") throw std::runtime_error(x.first+" cannot be given in stress units");
				x.second.unit = unit;
				*x.second.value *= std::abs(target_stress);
			}
		}
		resolve(unit);
	}
};

} // namespace

using lfg::fail;
using lfg::ok;

extern "C" int lfg_config_resolve(const char *text, char control, const char *control_value, lfg_params *out,
                                  double *time_end, double *strain_end, lfg_status *st)
{
	if (!text || !control_value || !out || (control != 'r' && control != 's'))
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	try {
		Resolver R;
		std::string num, suf;
		if (!get_suffix(control_value, num, suf)) throw std::runtime_error("the control value needs a unit suffix");
		double number = std::atof(num.c_str());
		R.defaults(suf);
		R.read(text);
		R.tag_strain();
		auto ln = R.longname.find(suf);
		if (ln == R.longname.end()) throw std::runtime_error("unknown unit suffix "+suf);
		const std::string scale = ln->second;
		if (control == 'r') R.rate_controlled(number, scale);
		else R.stress_controlled(number, scale);
		// exportForceAmplitudes + assertParameterCompatibility
		Params &p = R.p;
		R.repulsiveforce = R.input_values.count("repulsion") > 0;
		R.critical_load_on = R.input_values.count("critical_load") > 0;
		if (R.input_values.count("cohesion")) throw std::runtime_error("cohesion is not supported by this engine");
		const bool brownian = R.input_values.count("brownian") > 0;
		if (brownian && control != 'r')
			throw std::runtime_error("stress-controlled Brownian runs are not supported by this engine");
		if (brownian && p.integration_method != 1)
			throw std::runtime_error("Brownian simulation needs to use the Predictor-Corrector method.");
		if (R.input_values.count("hydro")) R.shear_rate = *R.input_values["hydro"].value;
		if (R.critical_load_on) p.friction_model = 2;
		// resolveTimeOrStrainParameters
		double te, se = -1;
		if (R.input_values["time_end"].unit == "strain") { te = -1; se = p.time_end; }
		else te = p.time_end;
		// System::setupParameters* (System.cpp:348-414)
		if (p.friction_model == 0) p.mu_static = 0;
		if (p.mu_dynamic < 0) p.mu_dynamic = p.mu_static;
		if (p.mu_rolling > 0 && p.friction_model == 0)
			throw std::runtime_error("rolling friction without sliding friction");
		bool repulsion_on = R.repulsiveforce;
		if (p.repulsive_length <= 0) { repulsion_on = false; p.repulsive_length = 0; }
		int lub = p.lubrication_model == "none" ? 0 : p.lubrication_model == "normal" ? 1
		          : p.lubrication_model == "tangential" ? 2 : -1;
		if (lub < 0) throw std::runtime_error("unknown lubrication_model "+p.lubrication_model);
		lfg_params o;
		std::memset(&o, 0, sizeof o);
		o.kn = p.kn; o.kt = p.kt;
		o.mu_static = p.mu_static; o.mu_dynamic = p.mu_dynamic;
		o.critical_load = p.critical_load; o.ft_max = p.ft_max;
		o.friction_model = p.friction_model;
		o.repulsion_on = repulsion_on ? 1 : 0; o.repulsion = p.repulsion;
		o.repulsive_length = p.repulsive_length; o.repulsive_max_length = p.repulsive_max_length;
		o.lubrication_model = lub;
		o.lub_reduce_parameter = p.lub_reduce_parameter; o.lub_max_gap = p.lub_max_gap;
		o.interaction_range = p.interaction_range;   // -1: the lubrication range (System.cpp:405-410)
		o.sd_coeff = p.simulation_mode == 31 ? 1e-6 : p.sd_coeff;
		o.contact_relaxation_time = p.contact_relaxation_time;
		o.contact_relaxation_time_tan = p.contact_relaxation_time_tan;
		o.disp_max = p.disp_max; o.dt = p.dt; o.dt_max = p.dt_max; o.dt_min = p.dt_min;
		o.fixed_dt = p.fixed_dt ? 1 : 0;
		o.integration_method = p.integration_method;
		o.control = control == 's' ? 1 : 0;
		o.shear_rate = R.shear_rate;
		o.target_stress = R.target_stress;
		// simple shear at unit rate (SimulationInit.cpp:615-630)
		const double Eh[6] = {0, 0, 0.5, 0, 0, 0}, Oh[3] = {0, 0.5, 0};
		std::memcpy(o.Ehat, Eh, sizeof Eh);
		std::memcpy(o.Ohat, Oh, sizeof Oh);
		o.init_strain_shear_rate_limit = 0;
		o.init_shear_rate_limit = 999;
		o.mu_rolling = p.mu_rolling; o.kr = p.kr;
		o.brownian = brownian ? p.brownian : 0;   // kT in hydro units (exportForceAmplitudes)
		o.seed = 0;
		*out = o;
		if (time_end) *time_end = te;
		if (strain_end) *strain_end = se;
		return ok(st);
	} catch (const std::exception &e) {
		return fail(st, LFG_ERR_BAD_ARG, 0, e.what());
	}
}

// Output units and switches (Simulation::setupNonDimensionalization,
// SimulationInit.cpp:287-295, 392-402, 455-472; Simulation::outputData's
// force_ratios[internal/output], Simulation.cpp:654-663): the output unit is
// the control value's scale; the internal one is "hydro" under rate
// control (non-Brownian) and the stress's unit under stress control.
extern "C" int lfg_config_output(const char *text, char control, const char *control_value, lfg_output_units *out,
                                 lfg_status *st)
{
	if (!text || !control_value || !out || (control != 'r' && control != 's'))
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	try {
		Resolver R;
		std::string num, suf;
		if (!get_suffix(control_value, num, suf)) throw std::runtime_error("the control value needs a unit suffix");
		double number = std::atof(num.c_str());
		R.defaults(suf);
		R.read(text);
		R.tag_strain();
		auto ln = R.longname.find(suf);
		if (ln == R.longname.end()) throw std::runtime_error("unknown unit suffix "+suf);
		const std::string scale = ln->second;
		if (control == 'r') R.rate_controlled(number, scale);
		else R.stress_controlled(number, scale);
		const std::string internal = control == 'r' ? std::string("hydro") : scale;
		auto it = R.force_ratios.find(internal+"/"+scale);
		if (it == R.force_ratios.end())
			throw std::runtime_error("cannot convert from \""+internal+"\" units to \""+scale+"\" units");
		lfg_output_units u;
		std::memset(&u, 0, sizeof u);
		std::snprintf(u.unit, sizeof u.unit, "%s", scale.c_str());
		u.internal_to_output = it->second;
		u.input_value = number;
		u.out_data_particle = R.p.out_data_particle;
		u.out_data_interaction = R.p.out_data_interaction;
		u.origin_zero_flow = R.p.origin_zero_flow;
		std::snprintf(u.out_particle_stress, sizeof u.out_particle_stress, "%s", R.p.out_particle_stress.c_str());
		*out = u;
		return ok(st);
	} catch (const std::exception &e) {
		return fail(st, LFG_ERR_BAD_ARG, 0, e.what());
	}
}
