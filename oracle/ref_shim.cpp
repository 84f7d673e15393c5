// TEST INFRASTRUCTURE ONLY: a C-callable shim over the reference's own CGS
// code (src/cgs_read.cpp, src/cgs_data.cpp, src/cgs.cpp, compiled unmodified
// by `make ref` into _ref/libsjref.so).  tests/golden/make_golden.py calls
// it to record what the reference answers; nothing in the product links it.
//
// It does three things a maintainer wiring bound_geom to include/sj.h does:
//   * parse a .geom file with the reference's scene (src/cgs.cpp:577);
//   * flatten each root composite_object into sj_csg_node postfix programs
//     with the integration guide's own code (copied
//     verbatim into _ref/guide_flatten.inc at build time), compiled against
//     the reference's cgs.hpp with the four accessors the guide asks for
//     (trans_mat, invert, the cylinder's r1_sq and r2_sq; oracle/guide_build.py);
//   * restate parse_susceptibilities (src/disp.cpp:418-454), which lives in
//     meep-dependent code, on the root's "susceptibilities" metadata.
// It also exposes composite_object::in (src/cgs.cpp:431-456) itself and the
// reference's fft (src/data_utils.cpp:413-427, the transform save_field_times
// applies to each monitor series), the answers the golden vectors record.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cgs.hpp"
#include "cgs_read.hpp"
#include "data_utils.hpp"
#include "sj.h"

namespace {

std::vector<scene*> g_scenes;

}  // namespace

// The integration guide's walk, verbatim (mat_copy and flatten).
#include "guide_flatten.inc"

namespace {

// um_to_l and fs_to_t (src/disp.cpp:5-22): lengths in um and times in fs to
// the scene's length units, scaled by the context's l_per_um
value shim_um_to_l(context& c, cgs_func f, parse_ercode& er) {
    value ret;
    if (f.n_args < 1) { er = E_LACK_TOKENS; return ret; }
    if (f.args[0].type != VAL_NUM) { er = E_BAD_TOKEN; return ret; }
    value l_per_um = c.lookup("l_per_um");
    if (l_per_um.type != VAL_NUM) { er = E_NOT_DEFINED; return ret; }
    return make_val_num(l_per_um.val.x * f.args[0].val.x);
}
value shim_fs_to_t(context& c, cgs_func f, parse_ercode& er) {
    value ret;
    if (f.n_args < 1) { er = E_LACK_TOKENS; return ret; }
    if (f.args[0].type != VAL_NUM) { er = E_BAD_TOKEN; return ret; }
    value l_per_um = c.lookup("l_per_um");
    if (l_per_um.type != VAL_NUM) { er = E_NOT_DEFINED; return ret; }
    return make_val_num(0.299792458 * l_per_um.val.x * f.args[0].val.x);
}

composite_object* root_of(int h, int r) {
    if (h < 0 || h >= (int)g_scenes.size() || !g_scenes[h]) return nullptr;
    std::vector<composite_object*> roots = g_scenes[h]->get_roots();
    if (r < 0 || r >= (int)roots.size()) return nullptr;
    return roots[r];
}

}  // namespace

extern "C" {

// Parse a .geom file; returns a handle >= 0, or -(1 + parse_ercode) on failure.
int sjref_load(const char* path) {
    parse_ercode er = E_SUCCESS;
    scene* s = new scene(path, &er);
    if (er != E_SUCCESS) {
        delete s;
        return -(1 + (int)er);
    }
    g_scenes.push_back(s);
    return (int)g_scenes.size() - 1;
}

// Parse with the context bound_geom gives a scene (restating
// context_from_settings, src/disp.cpp:28-50): pi, pml_thickness, sim_length,
// length = 2 pml + len, l_per_um, out_dir, um_to_l, fs_to_t, then the
// user options ("name=value;..." as --opts passes them).
int sjref_load_ctx(const char* path, double pml_thickness, double len, double um_scale, const char* opts) {
    context con;
    con.emplace("pi", make_val_num(M_PI));
    con.emplace("pml_thickness", make_val_num(pml_thickness));
    con.emplace("sim_length", make_val_num(len));
    con.emplace("length", make_val_num(2 * pml_thickness + len));
    con.emplace("l_per_um", make_val_num(um_scale));
    value tmp = make_val_str(".");
    con.emplace("out_dir", tmp);
    cleanup_val(&tmp);
    tmp = make_val_func("um_to_l", 1, &shim_um_to_l);
    con.emplace("um_to_l", tmp);
    cleanup_val(&tmp);
    tmp = make_val_func("fs_to_t", 1, &shim_fs_to_t);
    con.emplace("fs_to_t", tmp);
    cleanup_val(&tmp);
    if (opts && *opts) {
        line_buffer lb(opts, ';');
        con.read_from_lines(lb);
    }
    parse_ercode er = E_SUCCESS;
    scene* s = new scene(path, con, &er);
    if (er != E_SUCCESS) {
        delete s;
        return -(1 + (int)er);
    }
    g_scenes.push_back(s);
    return (int)g_scenes.size() - 1;
}

int sjref_n_roots(int h) {
    if (h < 0 || h >= (int)g_scenes.size() || !g_scenes[h]) return -1;
    return (int)g_scenes[h]->get_roots().size();
}

// Postfix program of root r; returns its node count (nothing is written when
// it exceeds cap), -1 for a bad handle or root.
int sjref_flatten(int h, int r, sj_csg_node* out, int cap) {
    composite_object* root = root_of(h, r);
    if (!root) return -1;
    std::vector<sj_csg_node> prog;
    flatten(root, CGS_COMPOSITE, mat3x3::id(), prog);
    if ((int)prog.size() <= cap) memcpy(out, prog.data(), prog.size() * sizeof(sj_csg_node));
    return (int)prog.size();
}

// The root's "eps" metadata, or def when it has none.
double sjref_root_eps(int h, int r, double def) {
    composite_object* root = root_of(h, r);
    if (!root || !root->has_metadata("eps")) return def;
    return root->fetch_metadata("eps").to_float();
}

// Susceptibilities of root r (restating parse_susceptibilities): returns the
// count (entries beyond cap are not written) or a negative parse error.
int sjref_root_poles(int h, int r, double* omega_0, double* gamma, double* sigma, int* drude, int cap) {
    composite_object* root = root_of(h, r);
    if (!root) return -1;
    if (!root->has_metadata("susceptibilities")) return 0;
    value val = root->fetch_metadata("susceptibilities");
    if (val.type != VAL_LIST) return 0;
    int n = 0;
    for (size_t i = 0; i < val.n_els; ++i) {
        value cur = val.val.l[i];
        if (cur.type != VAL_LIST || cur.n_els < 3) return -2;
        if (cur.val.l[0].type != VAL_NUM || cur.val.l[1].type != VAL_NUM || cur.val.l[2].type != VAL_NUM) return -3;
        int use_denom = 1;
        if (cur.n_els > 3) {
            const value& k = cur.val.l[3];
            if (k.type == VAL_NUM) {
                use_denom = k.val.x != 0.0;
            } else if (k.type == VAL_STR) {
                if (strcmp(k.val.s, "drude") == 0 || strcmp(k.val.s, "true") == 0) use_denom = 0;
                if (strcmp(k.val.s, "lorentz") == 0 || strcmp(k.val.s, "false") == 0) use_denom = 1;
            } else {
                return -3;
            }
        }
        if (n < cap) {
            omega_0[n] = cur.val.l[0].val.x;
            gamma[n] = cur.val.l[1].val.x;
            sigma[n] = cur.val.l[2].val.x;
            drude[n] = !use_denom;
        }
        ++n;
    }
    return n;
}

// fft of the series re + i im (n points): writes the result (its length is
// returned, at most cap complex values) as out[k][re, im].
int64_t sjref_fft(const double* re, const double* im, int64_t n, double* out, int64_t cap) {
    data_arr dat;
    make_data_arr_zeros(&dat, (_ulong)n);
    for (int64_t q = 0; q < n; ++q) {
        dat.buf[q].re = re[q];
        dat.buf[q].im = im[q];
    }
    data_arr r = fft(dat);
    const int64_t m = (int64_t)r.size;
    for (int64_t k = 0; k < m && k < cap; ++k) {
        out[2 * k] = r.buf[k].re;
        out[2 * k + 1] = r.buf[k].im;
    }
    cleanup_data_arr(&r);
    cleanup_data_arr(&dat);
    return m;
}

// composite_object::in of root r at n points (xyz interleaved).
int sjref_in(int h, int r, const double* pts, int64_t n, uint8_t* out) {
    composite_object* root = root_of(h, r);
    if (!root) return -1;
    for (int64_t q = 0; q < n; ++q) out[q] = (uint8_t)root->in(vec3(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]));
    return 0;
}

// A primitive built with the reference's own constructors, as its volume
// test builds them (src/main_test.cpp:1448-1459), and its in() at n points.
// kind 0: sphere(center, rad), a = {cx, cy, cz, rad}; kind 1: cylinder(center,
// height, r1, r2), a = {cx, cy, cz, height, r1, r2}; kind 2: plane(p1, p2,
// p3), a = the three points.
static void primitive_eval(object& obj, const double* pts, int64_t n, uint8_t* out) {
    for (int64_t q = 0; q < n; ++q) out[q] = (uint8_t)obj.in(vec3(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]));
}

int sjref_primitive_in(int kind, const double* a, const double* pts, int64_t n, uint8_t* out) {
    vec3 c(a[0], a[1], a[2]);
    if (kind == 0) {
        sphere obj(c, a[3]);
        primitive_eval(obj, pts, n, out);
    } else if (kind == 1) {
        cylinder obj(c, a[3], a[4], a[5]);
        primitive_eval(obj, pts, n, out);
    } else if (kind == 2) {
        vec3 p2(a[3], a[4], a[5]), p3(a[6], a[7], a[8]);
        plane obj(c, p2, p3);
        primitive_eval(obj, pts, n, out);
    } else {
        return -1;
    }
    return 0;
}

}  // extern "C"
