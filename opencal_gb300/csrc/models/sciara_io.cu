/*
 * sciara_io.cu -- the SCIARA-fv2 configuration reader: the reference
 * example's input files, so that its real inputs (e.g. the 2006 Etna
 * configuration it ships) run on the GPU through cal_sciara_run.
 *
 * Restates, for reading only:
 *   loadConfiguration  OpenCAL-OMP/examples/calomp_sciara-fv2/source/io.cpp:357-404
 *     <path>.cfg, else <path>_000000000000.cfg; the other files are the .cfg
 *     path without ".cfg" plus "_<name><suffix>"
 *     (configurationPathLib.cpp, ConfigurationFilePath)
 *   loadParameters     io.cpp:60-150: "key value" pairs in a fixed order,
 *     each key checked; the 12 physical parameters are kept
 *   LeggiGISInfo       GISInfo.cpp:11-52: ncols, nrows, xllcorner,
 *     yllcorner, cellsize, NODATA_value, then exactly ncols * nrows values
 *   VerificaGISInfo    GISInfo.cpp:54-62: every other grid matches the
 *     morphology's size, corner (within a cell) and cell size
 *   loadMorphology     io.cpp:248-271: Sz; Pc = cellsize
 *   loadVents + initVents  io.cpp:273-293, vent.cpp:15-31: every cell with
 *     id > 0 is a vent, in row-major order (x = column, y = row)
 *   loadEmissionRates + defineVents  vent.cpp:49-133, 184-190: [TIME] t,
 *     then [VENT_ID] id [EMISSION_RATE] rates... per vent, ending at [END];
 *     every vent id of the grid needs rates
 *   Thickness, Temperature, SolidifiedLavaThickness .stt: optional
 *     (io.cpp:388-398 reads them when present)
 * Vents whose rate lists differ in length are padded with zeros, which is
 * what the reference's TVent::thickness returns past the end of a list.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "opencal/calCommon.h"

namespace {

struct GisHeader {
    int ncols = 0, nrows = 0;
    double xll = 0, yll = 0, cell = 0, nodata = 0;
};

/* LeggiGISInfo: the six header keys, then the count of remaining values */
bool read_gis_header(FILE* f, GisHeader& h)
{
    static const char* keys[6] = {"ncols", "nrows", "xllcorner", "yllcorner", "cellsize", "NODATA_value"};
    char str[256];
    double v[6];
    for (int k = 0; k < 6; k++) {
        if (fscanf(f, "%255s", str) != 1 || strcmp(str, keys[k]) != 0)
            return false;
        if (fscanf(f, "%255s", str) != 1)
            return false;
        v[k] = atof(str);
    }
    h.ncols = (int)v[0];
    h.nrows = (int)v[1];
    h.xll = v[2];
    h.yll = v[3];
    h.cell = v[4];
    h.nodata = v[5];
    fpos_t pos;
    fgetpos(f, &pos);
    long long count = 0;
    while (fscanf(f, "%255s", str) == 1)
        count++;
    fsetpos(f, &pos);
    return h.ncols > 0 && h.nrows > 0 && count == (long long)h.ncols * h.nrows;
}

bool same_grid(const GisHeader& a, const GisHeader& m)
{
    return a.ncols == m.ncols && a.nrows == m.nrows && !(fabs(a.xll - m.xll) > m.cell) &&
           !(fabs(a.yll - m.yll) > m.cell) && a.cell == m.cell;
}

std::string file_path(const std::string& cfg, const char* name, const char* suffix)
{
    return cfg.substr(0, cfg.size() - 4) + "_" + name + suffix;
}

/* loadParameters: the keys in order, the 12 physical parameters kept */
bool read_parameters(const std::string& path, double* params)
{
    static const char* keys[17] = {"maximum_steps_(0_for_loop)", "stopping_threshold_(height)", "refreshing_step",
                                   "thickness_visual_threshold", "Pclock", "PTsol", "PTvent", "Pr(Tsol)",
                                   "Pr(Tvent)", "Phc(Tsol)", "Phc(Tvent)", "Pcool", "Prho", "Pepsilon", "Psigma",
                                   "Pcv", "algorithm"};
    FILE* f = fopen(path.c_str(), "r");
    if (!f)
        return false;
    char str[256];
    bool ok = true;
    for (int k = 0; k < 17 && ok; k++) {
        ok = fscanf(f, "%255s", str) == 1 && strcmp(str, keys[k]) == 0 && fscanf(f, "%255s", str) == 1;
        if (ok && k >= 4 && k < 16)
            params[k - 4] = atof(str);
    }
    fclose(f);
    return ok;
}

struct Vent {
    int x, y, id;
};

/* loadEmissionRates: [TIME] t, then per vent [VENT_ID] id [EMISSION_RATE] r... */
bool read_emission(const std::string& path, const std::vector<Vent>& vents, unsigned* emission_time,
                   std::vector<std::vector<double>>& rates_by_vent)
{
    FILE* f = fopen(path.c_str(), "r");
    if (!f)
        return false;
    char str[256];
    bool ok = fscanf(f, "%255s", str) == 1 && strcmp(str, "[TIME]") == 0 && fscanf(f, "%255s", str) == 1 &&
              atoi(str) >= 0;
    if (ok)
        *emission_time = (unsigned)atoi(str);
    std::vector<std::pair<int, std::vector<double>>> lists;
    bool done = false;
    if (ok && fscanf(f, "%255s", str) != 1)
        ok = false;
    while (ok && !done) {
        if (strcmp(str, "[VENT_ID]") != 0 || fscanf(f, "%255s", str) != 1 || atoi(str) < 0) {
            ok = false;
            break;
        }
        const int id = atoi(str);
        bool known = false;
        for (const Vent& v : vents)
            known = known || v.id == id;
        if (!known || fscanf(f, "%255s", str) != 1 || strcmp(str, "[EMISSION_RATE]") != 0 ||
            fscanf(f, "%255s", str) != 1 || atof(str) < 0) {
            ok = false;
            break;
        }
        std::vector<double> r;
        for (;;) {
            r.push_back(atof(str));
            if (fscanf(f, "%255s", str) != 1) {
                ok = false; /* the file ended before [END] */
                break;
            }
            if (strcmp(str, "[END]") == 0) {
                done = true;
                break;
            }
            if (strcmp(str, "[VENT_ID]") == 0)
                break;
        }
        lists.push_back(std::make_pair(id, r));
    }
    fclose(f);
    if (!ok)
        return false;
    rates_by_vent.clear();
    for (const Vent& v : vents) {
        const std::vector<double>* found = nullptr;
        for (const auto& l : lists)
            if (l.first == v.id) {
                found = &l.second;
                break;
            }
        if (!found)
            return false; /* defineVents: every vent needs its rates */
        rates_by_vent.push_back(*found);
    }
    return true;
}

/* an optional grid of the configuration; false when it exists but is not
 * valid for the morphology */
bool read_optional_grid(const std::string& path, const GisHeader& morph, double* out, int* present)
{
    *present = 0;
    FILE* f = fopen(path.c_str(), "r");
    if (!f)
        return true;
    GisHeader h;
    bool ok = read_gis_header(f, h) && same_grid(h, morph);
    char str[256];
    const long long n = (long long)morph.ncols * morph.nrows;
    for (long long c = 0; ok && c < n; c++) {
        ok = fscanf(f, "%255s", str) == 1;
        if (ok && out)
            out[c] = atof(str);
    }
    fclose(f);
    *present = ok ? 1 : 0;
    return ok;
}

struct Config {
    GisHeader morph;
    std::vector<Vent> vents;
    std::vector<std::vector<double>> rates;
    unsigned emission_time = 0;
    int nphases = 0;
};

int read_config(const char* path, Config& c, double* params, double* z, std::string* cfg_used = nullptr)
{
    /* the path as given, else with "_000000000000.cfg" appended (io.cpp:364-368) */
    std::string cfg(path);
    double p[12];
    if (!read_parameters(cfg, p)) {
        cfg += "_000000000000.cfg";
        if (!read_parameters(cfg, p))
            return CAL_ERROR_IO;
    }
    if (params) {
        memcpy(params, p, sizeof(p));
    }
    FILE* f = fopen(file_path(cfg, "Morphology", ".stt").c_str(), "r");
    if (!f)
        return CAL_ERROR_IO;
    bool ok = read_gis_header(f, c.morph);
    char str[256];
    const long long n = (long long)c.morph.ncols * c.morph.nrows;
    for (long long k = 0; ok && k < n; k++) {
        ok = fscanf(f, "%255s", str) == 1;
        if (ok && z)
            z[k] = atof(str);
    }
    fclose(f);
    if (!ok)
        return CAL_ERROR_IO;
    if (params)
        params[12] = c.morph.cell; /* Pc */
    f = fopen(file_path(cfg, "Vents", ".stt").c_str(), "r");
    if (!f)
        return CAL_ERROR_IO;
    GisHeader hv;
    ok = read_gis_header(f, hv) && same_grid(hv, c.morph);
    c.vents.clear();
    for (long long k = 0; ok && k < n; k++) {
        ok = fscanf(f, "%255s", str) == 1;
        const int id = ok ? atoi(str) : 0;
        if (id > 0)
            c.vents.push_back(Vent{(int)(k % c.morph.ncols), (int)(k / c.morph.ncols), id});
    }
    fclose(f);
    if (!ok)
        return CAL_ERROR_IO;
    if (!read_emission(file_path(cfg, "EmissionRate", ".txt"), c.vents, &c.emission_time, c.rates))
        return CAL_ERROR_IO;
    c.nphases = 0;
    for (const auto& r : c.rates)
        c.nphases = (int)r.size() > c.nphases ? (int)r.size() : c.nphases;
    if (cfg_used)
        *cfg_used = cfg;
    return CAL_SUCCESS;
}

} // namespace

/* Sizes of a SCIARA-fv2 configuration (see cal_sciara_read). */
extern "C" int cal_sciara_read_sizes(const char* path, int* rows, int* cols, int* nvents, int* nphases)
{
    Config c;
    const int rc = read_config(path, c, nullptr, nullptr);
    if (rc != CAL_SUCCESS)
        return rc;
    *rows = c.morph.nrows;
    *cols = c.morph.ncols;
    *nvents = (int)c.vents.size();
    *nphases = c.nphases;
    return CAL_SUCCESS;
}

/* Reads a SCIARA-fv2 configuration.  params: the 12 .cfg parameters and Pc
 * (13 doubles, cal_sciara_run's order); z: rows x cols; vent_xy: (x, y) per
 * vent in the reference's vent order; rates: nvents x nphases; slt, st, msl
 * (optional, rows x cols each, may be NULL): the initial thickness,
 * temperature and solidified thickness when their files exist, with
 * present[3] saying which did (absent ones are left untouched). */
extern "C" int cal_sciara_read(const char* path, double* params, double* z, int* vent_xy, double* rates,
                               unsigned* emission_time, double* slt, double* st, double* msl, int* present)
{
    Config c;
    std::string cfg;
    int rc = read_config(path, c, params, z, &cfg);
    if (rc != CAL_SUCCESS)
        return rc;
    for (size_t v = 0; v < c.vents.size(); v++) {
        vent_xy[2 * v] = c.vents[v].x;
        vent_xy[2 * v + 1] = c.vents[v].y;
        for (int p = 0; p < c.nphases; p++)
            rates[v * c.nphases + p] = p < (int)c.rates[v].size() ? c.rates[v][p] : 0.0;
    }
    *emission_time = c.emission_time;
    const char* names[3] = {"Thickness", "Temperature", "SolidifiedLavaThickness"};
    double* outs[3] = {slt, st, msl};
    int have[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++)
        if (!read_optional_grid(file_path(cfg, names[k], ".stt"), c.morph, outs[k], &have[k]))
            return CAL_ERROR_IO;
    if (present)
        memcpy(present, have, sizeof(have));
    return CAL_SUCCESS;
}
