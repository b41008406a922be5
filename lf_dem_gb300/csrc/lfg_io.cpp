// lfg_io.cpp -- LF_DEM's checkpoint formats, so a suspension advanced by the
// engine can be saved and restarted with the reference's own files:
//  - binary configuration (conf_*.dat): Simulation::outputConfigurationBinary
//    (Simulation.cpp:513-600) and readBinaryBaseConfiguration /
//    readContactStatesBStream (Configuration.h:67-120, 212-245).  Version 2
//    has the label (-1, 2); the unlabelled old format starts with np, and its
//    contacts may use unsigned short particle numbers, recognised as the
//    reference does: a first particle number above np means unsigned short;
//  - state file (chk_*.dat): State::outputStateBinary / readBasicCheckpoint
//    (States.cpp:9-66): format 1, strain, time, time in simulation units.
// Plain host I/O; no device call.
#include <cstdio>
#include <cstring>
#include <vector>

#include "lfg_internal.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);
int ok(lfg_status *st);
}
using lfg::fail;
using lfg::ok;

namespace {
struct File {
	FILE *f = nullptr;
	explicit File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
	~File() { if (f) std::fclose(f); }
	template <typename V> bool put(const V &v) { return std::fwrite(&v, sizeof v, 1, f) == 1; }
	template <typename V> bool get(V &v) { return std::fread(&v, sizeof v, 1, f) == 1; }
};
} // namespace

extern "C" {

int lfg_conf_write_binary(const char *path, int np, double vf, double lx, double ly, double lz,
                          const double *le_disp, const double *pos, const double *radius, int ncont,
                          const int32_t *p0, const int32_t *p1, const double *disp_tan, const double *disp_rolling,
                          lfg_status *st)
{
	if (!path || np <= 0 || !pos || !radius || ncont < 0 || (ncont > 0 && (!p0 || !p1 || !disp_tan)))
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	File F(path, "wb");
	if (!F.f) return fail(st, LFG_ERR_BAD_ARG, 0, "cannot open the configuration file for writing");
	bool w = F.put((int)-1) && F.put((int)2) && F.put(np) && F.put(vf) && F.put(lx) && F.put(ly) && F.put(lz) &&
	         F.put(le_disp ? le_disp[0] : 0.0) && F.put(le_disp ? le_disp[1] : 0.0);
	for (int i = 0; w && i < np; i++)
		w = F.put(pos[3*i]) && F.put(pos[3*i+1]) && F.put(pos[3*i+2]) && F.put(radius[i]);
	w = w && F.put((unsigned int)ncont);
	for (int c = 0; w && c < ncont; c++) {
		w = F.put((unsigned int)p0[c]) && F.put((unsigned int)p1[c]);
		for (int k = 0; w && k < 3; k++) w = F.put(disp_tan[3*c+k]);
		for (int k = 0; w && k < 3; k++) w = F.put(disp_rolling ? disp_rolling[3*c+k] : 0.0);
	}
	if (!w) return fail(st, LFG_ERR_BAD_ARG, 0, "write error");
	return ok(st);
}

// Reads a binary base configuration.  Call once with NULL arrays for np and
// ncont, then with arrays of 3 np (pos), np (radius), ncont (p0, p1) and
// 3 ncont (disp_tan, disp_rolling) values.  meta (may be NULL): vf, lx, ly,
// lz, le_disp x, le_disp y.  *format: 2 (labelled) or 1 (unlabelled).
int lfg_conf_read_binary(const char *path, int *np_out, int *ncont_out, int *format, double *meta, double *pos,
                         double *radius, int32_t *p0, int32_t *p1, double *disp_tan, double *disp_rolling,
                         lfg_status *st)
{
	if (!path || !np_out || !ncont_out) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	File F(path, "rb");
	if (!F.f) return fail(st, LFG_ERR_BAD_ARG, 0, "cannot open the configuration file");
	int first = 0, fmt = 1, np = 0;
	if (!F.get(first)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
	if (first == -1) {
		if (!F.get(fmt) || !F.get(np)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
		if (fmt != 2) return fail(st, LFG_ERR_BAD_ARG, fmt, "only the base binary format (2) is supported");
	} else {
		np = first;
	}
	if (np <= 0) return fail(st, LFG_ERR_BAD_ARG, np, "bad particle count");
	double m[6];
	for (double &v : m)
		if (!F.get(v)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
	std::vector<double> P(4*(size_t)np);
	if (std::fread(P.data(), sizeof(double), P.size(), F.f) != P.size())
		return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
	unsigned int ncont = 0;
	if (!F.get(ncont)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
	long cpos = std::ftell(F.f);
	std::vector<int32_t> a(ncont), b(ncont);
	std::vector<double> d(6*(size_t)ncont);
	bool ushort_format = false;
	for (unsigned int c = 0; c < ncont; c++) {
		unsigned int q0 = 0, q1 = 0;
		if (!F.get(q0)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
		if (q0 > (unsigned)np) { ushort_format = true; break; }   // Configuration.h:78-84
		if (!F.get(q1) || std::fread(&d[6*c], sizeof(double), 6, F.f) != 6)
			return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
		a[c] = (int32_t)q0;
		b[c] = (int32_t)q1;
	}
	if (ushort_format) {
		std::fseek(F.f, cpos, SEEK_SET);
		for (unsigned int c = 0; c < ncont; c++) {
			unsigned short q0 = 0, q1 = 0;
			if (!F.get(q0) || !F.get(q1) || std::fread(&d[6*c], sizeof(double), 6, F.f) != 6)
				return fail(st, LFG_ERR_BAD_ARG, 0, "truncated configuration file");
			a[c] = q0;
			b[c] = q1;
		}
	}
	*np_out = np;
	*ncont_out = (int)ncont;
	if (format) *format = first == -1 ? 2 : 1;
	if (meta) std::memcpy(meta, m, sizeof m);
	if (pos && radius)
		for (int i = 0; i < np; i++) {
			for (int k = 0; k < 3; k++) pos[3*i+k] = P[4*(size_t)i+k];
			radius[i] = P[4*(size_t)i+3];
		}
	for (unsigned int c = 0; c < ncont; c++) {
		if (p0) p0[c] = a[c];
		if (p1) p1[c] = b[c];
		for (int k = 0; k < 3; k++) {
			if (disp_tan) disp_tan[3*c+k] = d[6*c+k];
			if (disp_rolling) disp_rolling[3*c+k] = d[6*c+3+k];
		}
	}
	return ok(st);
}

int lfg_checkpoint_write(const char *path, double strain, double time, double time_in_simulation_units,
                         lfg_status *st)
{
	if (!path) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	File F(path, "wb");
	if (!F.f) return fail(st, LFG_ERR_BAD_ARG, 0, "cannot open the state file for writing");
	if (!(F.put((int)1) && F.put(strain) && F.put(time) && F.put(time_in_simulation_units)))
		return fail(st, LFG_ERR_BAD_ARG, 0, "write error");
	return ok(st);
}

int lfg_checkpoint_read(const char *path, double *strain, double *time, double *time_in_simulation_units,
                        lfg_status *st)
{
	if (!path) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	File F(path, "rb");
	if (!F.f) return fail(st, LFG_ERR_BAD_ARG, 0, "cannot open the state file");
	int fmt = 0;
	double a = 0, b = 0, c = 0;
	if (!F.get(fmt)) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated state file");
	if (fmt != 1) return fail(st, LFG_ERR_BAD_ARG, fmt, "only the basic state format (1) is supported");
	if (!(F.get(a) && F.get(b) && F.get(c))) return fail(st, LFG_ERR_BAD_ARG, 0, "truncated state file");
	if (strain) *strain = a;
	if (time) *time = b;
	if (time_in_simulation_units) *time_in_simulation_units = c;
	return ok(st);
}

} // extern "C"
