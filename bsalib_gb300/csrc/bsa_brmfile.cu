// bsa_brmfile.cu -- the response-bispectrum export files of bsa_Run: the reference's visual mode
// (bsa_enableVisualMode / bsa_setVisualIndexes, src/bsa/BsaLibImpl.F90:119-144, set up at
// :183-233) and its base export mode (bsa_setBRMExportDefaultMode, :1919-1932).
//
// File layout (exportBRM_baseHeaderWriter_internal_ / exportBRM_base_internal_, :1852-1913;
// the reference opens the file for unformatted STREAM access, src/IO/BsaIO.F90:233-241, so the
// values follow one another with no record markers; little-endian int32 / float32):
//   header, once:  int32 nm, int32 modes[nm], int32 ncomb, int32 ispsym, int32 nzones,
//                  int32 npts   (written as nm, then, in visual mode, replaced by the total
//                                number of points exported, writeNTotPtsToBispUn_, :1832-1845)
//   per zone:      int32 zone id (1 rectangle), int32 nI, int32 nJ
//   per point:     float32 f1, float32 f2, float32 value[ncomb]
// Visual mode, modal (bsacl "modal" true): nm = 3, modes = the three visual indexes, ncomb = 1,
// value = the response bispectrum of that modal combination; files bsaexport_cls.brm (the
// Classic grid as one nI = nJ = NFREQS zone, f1 fastest) and bsaexport_msh.brm (the Mesher zones,
// each zone's BRM lattice).  Visual mode, nodal: nm = 2, modes = (node, DOF), ncomb = 1, value =
// the nodal bispectrum getBRN (:1764-1800) of DOF (node - 1) NLIBS + DOF, Mesher only (the Classic
// analysis exports the modal form only, BsaClassicImpl.F90:158); files bsaexport_msh.brn.
// Base export mode (not visual): nm = the kept modes, modes = their ids, ncomb = dim_bisp, every
// combination per point, Mesher only (the Classic analysis exports in visual mode only).
//
// Reference quirks kept: getBRN_full_scalar_ reads the mode of the second index for the first
// (m = MODES(in), :1793), so the nodal value is sum phi_n phi_n phi_o B(m, n, o) over m, n, o;
// the npts record is only rewritten in visual mode.  Not kept: in base mode the reference writes
// to a unit it never opened (the files are opened in visual mode only, :188-222); here the base
// export goes to bsaexport_msh.brm.  Files are created in the working directory, as the
// reference opens them by bare name.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

struct BrmSink {
    FILE *fh = nullptr;
    long npts_pos = 0;
    int ncomb = 0;
    int kind = 0;            // 0 every combination, 1 one modal combination, 2 nodal (BRN)
    long long vis = 0;       // modal combination (0-based), kind 1
    std::vector<double> w;   // BRN weight of every combination, kind 2
    std::vector<float> row;  // one point's float32 record
    long long written = 0;
};

namespace {
bool put_i32(FILE *fh, int v) { return std::fwrite(&v, sizeof v, 1, fh) == 1; }
}  // namespace

// Whether this analysis writes an export file: the Classic grid in modal visual mode, the
// Mesher zones in visual mode or in base export mode.
bool Engine::brm_file_wanted(bool classic) const {
    if (!set.ibisp) return false;
    if (classic) return visual && visual_modal;
    return visual || brm_export_mode == 1;
}

int Engine::brm_file_open(bool classic, int nzones) {
    brm_file_close(-1);
    if (!brm_file_wanted(classic)) return BSA_OK;
    const int nm = nme;
    const long long nb = dim_bisp();
    BrmSink s;
    std::vector<int> modes_rec;
    if (visual) {
        if (visual_modal) {
            for (int k = 0; k < 3; ++k)
                if (visual_idx[k] < 1 || visual_idx[k] > nm)
                    return fail(BSA_ERR_ARG, "visual index %d of %d kept modes", visual_idx[k], nm);
            s.kind = 1;
            s.vis = set.onlyd ? visual_idx[0] - 1
                              : (long long)(visual_idx[2] - 1) * nm * nm + (long long)(visual_idx[1] - 1) * nm +
                                    (visual_idx[0] - 1);
            modes_rec.assign(visual_idx, visual_idx + 3);
        } else {
            if (visual_idx[0] < 1 || visual_idx[0] > in.nn) return fail(BSA_ERR_ARG, "Node index exceeds max n. of nodes");
            if (visual_idx[1] < 1 || visual_idx[1] > in.nlibs)
                return fail(BSA_ERR_ARG, "DOF index exceeds max n. of DOFs per node");
            if (!in.phi) return fail(BSA_ERR_UNSUPPORTED, "the nodal export needs the modal matrix");
            const long long dof = (long long)(visual_idx[0] - 1) * in.nlibs + (visual_idx[1] - 1);
            const int nd = in.phi_ndofs;
            if (dof >= nd) return fail(BSA_ERR_ARG, "visual DOF %lld outside the modal matrix", dof + 1);
            auto phi = [&](int im) { return in.phi[(size_t)dof + (size_t)nd * (modes[im] - 1)]; };
            s.kind = 2;
            s.w.resize((size_t)nb);
            if (set.onlyd) {
                for (int im = 0; im < nm; ++im) s.w[im] = phi(im) * phi(im) * phi(im);
            } else {
                for (int io = 0; io < nm; ++io)
                    for (int in_ = 0; in_ < nm; ++in_)
                        for (int im = 0; im < nm; ++im)  // m = MODES(in), as the reference reads it
                            s.w[(size_t)im + (size_t)nm * in_ + (size_t)nm * nm * io] = phi(in_) * phi(in_) * phi(io);
            }
            modes_rec.assign(visual_idx, visual_idx + 2);
        }
        s.ncomb = 1;
    } else {
        s.kind = 0;
        s.ncomb = (int)nb;
        modes_rec.assign(modes.begin(), modes.end());
    }
    const char *name = classic ? "bsaexport_cls.brm"
                               : (visual && !visual_modal ? "bsaexport_msh.brn" : "bsaexport_msh.brm");
    s.fh = std::fopen(name, "wb");
    if (!s.fh) return fail(BSA_ERR_ARG, "cannot create the export file %s", name);
    bool ok = put_i32(s.fh, (int)modes_rec.size());
    for (int m : modes_rec) ok = ok && put_i32(s.fh, m);
    ok = ok && put_i32(s.fh, s.ncomb) && put_i32(s.fh, set.bispsym) && put_i32(s.fh, nzones);
    s.npts_pos = std::ftell(s.fh);
    ok = ok && put_i32(s.fh, (int)modes_rec.size());
    if (!ok) {
        std::fclose(s.fh);
        return fail(BSA_ERR_ARG, "cannot write the export file %s", name);
    }
    s.row.resize((size_t)s.ncomb + 2);
    brm_sink = new BrmSink(std::move(s));
    return BSA_OK;
}

int Engine::brm_file_zone(int id, int nI, int nJ) {
    if (!brm_sink) return BSA_OK;
    if (!(put_i32(brm_sink->fh, id) && put_i32(brm_sink->fh, nI) && put_i32(brm_sink->fh, nJ)))
        return fail(BSA_ERR_ARG, "cannot write the export file");
    return BSA_OK;
}

int Engine::emit_brm(int npts, const double *f1, const double *f2, const double *brm) {
    if (export_fn) export_fn(npts, f1, f2, brm, export_user);
    if (!brm_sink) return BSA_OK;
    BrmSink &s = *brm_sink;
    const long long nb = dim_bisp();
    for (int p = 0; p < npts; ++p) {
        const double *b = brm + (size_t)p * nb;
        s.row[0] = (float)f1[p];
        s.row[1] = (float)f2[p];
        if (s.kind == 0) {
            for (long long x = 0; x < nb; ++x) s.row[2 + x] = (float)b[x];
        } else if (s.kind == 1) {
            s.row[2] = (float)b[s.vis];
        } else {
            double v = 0.0;
            for (long long x = 0; x < nb; ++x) v += s.w[x] * b[x];
            s.row[2] = (float)v;
        }
        if (std::fwrite(s.row.data(), sizeof(float), s.row.size(), s.fh) != s.row.size())
            return fail(BSA_ERR_ARG, "cannot write the export file");
    }
    s.written += npts;
    return BSA_OK;
}

// total < 0: abandon (close as is).  In visual mode the npts record receives the total.
int Engine::brm_file_close(long long total) {
    if (!brm_sink) return BSA_OK;
    BrmSink *s = brm_sink;
    brm_sink = nullptr;
    bool ok = true;
    if (total >= 0 && visual) {
        ok = std::fseek(s->fh, s->npts_pos, SEEK_SET) == 0 && put_i32(s->fh, (int)total);
    }
    ok = (std::fclose(s->fh) == 0) && ok;
    delete s;
    if (!ok && total >= 0) return fail(BSA_ERR_ARG, "cannot write the export file");
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" {

int bsa_enableVisualMode(void) {
    if (eng().halted) return BSA_ERR_STATE;
    eng().visual = true;
    return BSA_OK;
}

int bsa_setVisualIndexes(const int *indexes, int modal) {
    if (eng().halted) return BSA_ERR_STATE;
    if (!indexes) return eng().fail(BSA_ERR_ARG, "null visual indexes");
    for (int k = 0; k < 3; ++k) eng().visual_idx[k] = indexes[k];
    eng().visual_modal = modal != 0;
    return BSA_OK;
}

int bsa_setBRMExportDefaultMode(int imode) {
    if (eng().halted) return BSA_ERR_STATE;
    // BSA_EXPORT_BRM_MODE_NONE (0) leaves the setting as it is, any other value selects the
    // base mode (BsaLibImpl.F90:1919-1932: an unknown mode warns and sets the base mode)
    if (imode != 0) eng().brm_export_mode = 1;
    return BSA_OK;
}

}  // extern "C"
