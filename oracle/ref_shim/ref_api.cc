/*
 * ref_api.cc -- a C ABI over the reference's own codec classes, compiled from
 * the unmodified reference sources against the shim headers in this folder.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's pin).  It is built by
 * `make -C oracle ref` into oracle/_ref/libpvvc_ref.so when the reference
 * tree is present, and used to validate the C restatement (pvvc_oracle.c)
 * and to generate the committed golden fixtures (tests/golden/).
 *
 * Classes driven here: vvc::common::RLGREncoder/RLGRDecoder and
 * ZstdEncoder/ZstdDecoder (src/common/entropy_codec.cc),
 * vvc::octree::RAHTOctree (src/octree/raht_octree.cc),
 * vvc::octree::InvertRAHTOctree (src/octree/invert_raht_octree.cc),
 * vvc::io::SaveSlice/LoadSlice/ChangeSliceToFrame (src/io/slice_io.cc).
 */
#include <cstring>
#include <memory>
#include <vector>

#include "common/entropy_codec.h"
#include "io/slice_io.h"
#include "octree/octree.h"

// GoPEncoding keeps its interpolated colours private: this test driver reads
// them through a public view of the class declaration (the reference's
// source is compiled unchanged).  Standard headers first, so that only the
// reference's declarations see the redefinition.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <mutex>
#include <numeric>
#include <queue>
#include <thread>
#define private public
#include "patch/patch.h"
#undef private

using namespace vvc;

// registration::ICP is implemented with PCL's ICP (src/registration/icp.cc),
// which is not available here.  patch_fitting.cc names it only in
// PatchFitting::AddPatch, which this driver never calls; these definitions
// let the library link, and Align fails loudly if it is ever reached.
vvc::registration::ICP::ICP() : vvc::registration::ICPBase{}, icp_{nullptr} {}
void vvc::registration::ICP::Align() { throw __EXCEPT__(ERROR_OCCURED); }

namespace {
common::PVVCParam_t::Ptr make_params(int zstd_level) {
    auto p = std::make_shared<common::PVVCParam_t>();
    p->octree.resolution = 1.0f;
    p->zstd_level = zstd_level;
    p->thread_num = 1;
    return p;
}
}  // namespace

extern "C" {

/* ---- RLGR ---- */
long ref_rlgr_encode(const int64_t* sym, size_t n, uint8_t* out, size_t cap) {
    try {
        auto data = std::make_shared<std::vector<common::FIX_DATA_INT>>(sym, sym + n);
        common::RLGREncoder enc;
        enc.Encode(data);
        auto r = enc.GetResult();
        if (r->size() > cap) return -2;
        if (!r->empty()) std::memcpy(out, r->data(), r->size());
        return (long)r->size();
    } catch (const common::Exception&) {
        return -1;
    }
}

/* Decodes and returns how many symbols the decoder produced (it may exceed
 * nsym by a run's overshoot); copies min(produced, nsym). */
long ref_rlgr_decode(const uint8_t* in, size_t nbytes, size_t nsym, int64_t* out) {
    try {
        auto data = std::make_shared<std::vector<uint8_t>>(in, in + nbytes);
        common::RLGRDecoder dec;
        dec.Decode(data, (int)nsym);
        auto r = dec.GetResult();
        size_t m = r->size() < nsym ? r->size() : nsym;
        if (m) std::memcpy(out, r->data(), m * sizeof(int64_t));
        return (long)r->size();
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- zstd wrappers (entropy_codec.cc:289-373) ---- */
long ref_zstd_encode(const uint8_t* in, size_t n, int level, uint8_t* out, size_t cap) {
    try {
        common::ZstdEncoder enc;
        enc.SetParams(make_params(level));
        enc.Encode(std::make_shared<std::vector<uint8_t>>(in, in + n));
        auto r = enc.GetResult();
        if (r->size() > cap) return -2;
        std::memcpy(out, r->data(), r->size());
        return (long)r->size();
    } catch (const common::Exception&) {
        return -1;
    }
}

long ref_zstd_decode(const uint8_t* in, size_t n, uint8_t* out, size_t cap) {
    try {
        common::ZstdDecoder dec;
        dec.Decode(std::make_shared<std::vector<uint8_t>>(in, in + n));
        auto r = dec.GetResult();
        if (r->size() > cap) return -2;
        std::memcpy(out, r->data(), r->size());
        return (long)r->size();
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- encoder octree + RAHT ---- */
struct ref_encoder {
    octree::RAHTOctree tree;
    pcl::PointCloud<pcl::PointXYZRGB>::Ptr cloud;
};

void* ref_encoder_new(const float* xyz, size_t n) {
    try {
        auto* e = new ref_encoder();
        e->cloud.reset(new pcl::PointCloud<pcl::PointXYZRGB>());
        for (size_t i = 0; i < n; ++i) {
            pcl::PointXYZRGB p;
            p.x = xyz[3 * i];
            p.y = xyz[3 * i + 1];
            p.z = xyz[3 * i + 2];
            e->cloud->push_back(p);
        }
        e->tree.SetParams(make_params(22));
        e->tree.SetSourceCloud(e->cloud);
        e->tree.MakeTree();
        return e;
    } catch (const common::Exception&) {
        return nullptr;
    }
}

void ref_encoder_free(void* h) { delete static_cast<ref_encoder*>(h); }

long ref_encoder_geometry(void* h, uint8_t* out, size_t cap) {
    auto r = static_cast<ref_encoder*>(h)->tree.GetOctree();
    if (r->size() > cap) return -2;
    std::memcpy(out, r->data(), r->size());
    return (long)r->size();
}

/* yuv: n x 3 per input point; coef_out: leaf_count x 3 in stream order. */
long ref_encoder_raht(void* h, const float* yuv, size_t n, float* coef_out, size_t cap_leaves) {
    try {
        auto* e = static_cast<ref_encoder*>(h);
        auto colors = std::make_shared<std::vector<common::ColorYUV>>();
        for (size_t i = 0; i < n; ++i) colors->emplace_back(yuv[3 * i], yuv[3 * i + 1], yuv[3 * i + 2], true);
        e->tree.SetSourceColors(colors);
        e->tree.RAHT();
        auto r = e->tree.GetRAHTResult();
        if (r->size() > cap_leaves) return -2;
        for (size_t i = 0; i < r->size(); ++i) {
            coef_out[3 * i] = r->at(i).y;
            coef_out[3 * i + 1] = r->at(i).u;
            coef_out[3 * i + 2] = r->at(i).v;
        }
        return (long)r->size();
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- decoder ---- */
struct ref_decoder {
    octree::InvertRAHTOctree tree;
    common::Patch last;
};

void* ref_decoder_new(void) {
    auto* d = new ref_decoder();
    d->tree.SetParams(make_params(22));
    return d;
}

void ref_decoder_free(void* h) { delete static_cast<ref_decoder*>(h); }

/* mv is column-major (as a Slice holds it).  Payloads as stored in a slice
 * (possibly zstd frames, per the type bits). */
int ref_decoder_set_slice(void* h, uint8_t type, int timestamp, int index, uint64_t size, uint8_t qp, const float* mv_colmajor,
                          const uint8_t* geo, size_t gsz, const uint8_t* col, size_t csz) {
    try {
        auto* d = static_cast<ref_decoder*>(h);
        common::Slice s;
        s.type = type;
        s.timestamp = timestamp;
        s.index = index;
        s.size = size;
        s.qp = qp;
        std::memcpy(s.mv.d, mv_colmajor, 16 * sizeof(float));
        if (geo && gsz) s.geometry = std::make_shared<std::vector<uint8_t>>(geo, geo + gsz);
        if (col && csz) s.color = std::make_shared<std::vector<uint8_t>>(col, col + csz);
        d->tree.SetSlice(s);
        d->last = d->tree.GetPatch();
        return 0;
    } catch (const common::Exception&) {
        return -1;
    }
}

/* Points of the last decoded patch: pre-transform xyz and rgb as the
 * reference casts it. */
long ref_decoder_get_patch(void* h, float* xyz, uint8_t* rgb, size_t cap) {
    auto* d = static_cast<ref_decoder*>(h);
    if (!d->last.cloud) return -1;
    size_t n = d->last.cloud->size();
    if (n > cap) return -2;
    for (size_t i = 0; i < n; ++i) {
        const auto& p = d->last.cloud->at(i);
        xyz[3 * i] = p.x;
        xyz[3 * i + 1] = p.y;
        xyz[3 * i + 2] = p.z;
        rgb[3 * i] = p.r;
        rgb[3 * i + 1] = p.g;
        rgb[3 * i + 2] = p.b;
    }
    return (long)n;
}

/* ---- slice / frame files ---- */
int ref_save_slice(const char* path, uint8_t type, int timestamp, int index, uint64_t size, uint8_t qp, const float* mv_colmajor,
                   const uint8_t* geo, size_t gsz, const uint8_t* col, size_t csz) {
    try {
        common::Slice s;
        s.type = type;
        s.timestamp = timestamp;
        s.index = index;
        s.size = size;
        s.qp = qp;
        std::memcpy(s.mv.d, mv_colmajor, 16 * sizeof(float));
        if (geo && gsz) s.geometry = std::make_shared<std::vector<uint8_t>>(geo, geo + gsz);
        if (col && csz) s.color = std::make_shared<std::vector<uint8_t>>(col, col + csz);
        return io::SaveSlice(s, path);
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- GoPEncoding::Encode (src/patch/GoP_encoding.cc:97-210) on one patch's
 * GoP: the fitting cloud (n points; its colours are not used) and nf source
 * patches (xyz + rgb).  k = patch.interpolation_num.  Writes the interpolated
 * colours patch_colors_ (nf x n x YUV; later frames as residuals), the
 * geometry payload of slice 0 and each slice's colour payload, zstd undone
 * where the encoder kept the compressed form.  Returns 0, or -1 / -2. */
int ref_gop_encode(const float* fit_xyz, size_t n, int nf, const float* const* src_xyz, const uint8_t* const* src_rgb,
                   const size_t* src_n, int k, int qp_i, int qp_p, float* colors_out, uint8_t* geo_out, size_t geo_cap,
                   size_t* geo_len, uint8_t* col_out, size_t col_cap, size_t* col_len) {
    try {
        auto prm = std::make_shared<common::PVVCParam_t>();
        prm->octree.resolution = 1.0f;
        prm->zstd_level = 1;
        prm->thread_num = 1;
        prm->patch.interpolation_num = k;
        prm->slice.qp_i = (uint8_t)qp_i;
        prm->slice.qp_p = (uint8_t)qp_p;
        patch::GoPEncoding enc;
        enc.SetParams(prm);
        pcl::PointCloud<pcl::PointXYZRGB>::Ptr fit(new pcl::PointCloud<pcl::PointXYZRGB>());
        fit->resize(n);
        for (size_t i = 0; i < n; ++i) {
            (*fit)[i].x = fit_xyz[3 * i];
            (*fit)[i].y = fit_xyz[3 * i + 1];
            (*fit)[i].z = fit_xyz[3 * i + 2];
        }
        enc.SetFittingCloud(fit);
        std::vector<common::Patch> pats(nf);
        for (int f = 0; f < nf; ++f) {
            pats[f].cloud.reset(new pcl::PointCloud<pcl::PointXYZRGB>());
            pats[f].cloud->resize(src_n[f]);
            for (size_t i = 0; i < src_n[f]; ++i) {
                pcl::PointXYZRGB& q = (*pats[f].cloud)[i];
                q.x = src_xyz[f][3 * i];
                q.y = src_xyz[f][3 * i + 1];
                q.z = src_xyz[f][3 * i + 2];
                q.r = src_rgb[f][3 * i];
                q.g = src_rgb[f][3 * i + 1];
                q.b = src_rgb[f][3 * i + 2];
            }
            pats[f].timestamp = f;
            pats[f].index = 0;
        }
        enc.SetSourcePatches(pats);
        enc.Encode();
        for (int f = 0; f < nf; ++f)
            for (size_t i = 0; i < n; ++i) {
                const common::ColorYUV& c = enc.patch_colors_[f]->at(i);
                colors_out[(f * n + i) * 3] = c.y;
                colors_out[(f * n + i) * 3 + 1] = c.u;
                colors_out[(f * n + i) * 3 + 2] = c.v;
            }
        auto raw = [](uint8_t type, uint8_t bit, const std::shared_ptr<std::vector<uint8_t>>& b) {
            if (!(type & bit)) return *b;
            common::ZstdDecoder dec;
            dec.Decode(b);
            return *dec.GetResult();
        };
        std::vector<common::Slice> res = enc.GetResults();
        const std::vector<uint8_t> geo = raw(res[0].type, 0x08, res[0].geometry);
        if (geo.size() > geo_cap) return -2;
        std::memcpy(geo_out, geo.data(), geo.size());
        *geo_len = geo.size();
        size_t off = 0;
        for (int f = 0; f < nf; ++f) {
            const std::vector<uint8_t> c = raw(res[f].type, 0x10, res[f].color);
            if (off + c.size() > col_cap) return -2;
            std::memcpy(col_out + off, c.data(), c.size());
            col_len[f] = c.size();
            off += c.size();
        }
        return 0;
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- ICPBase::CloudMSE (src/registration/registration_base.cc:114-158) of
 * cloud a (the transformed source) against cloud b (the target); a derived
 * class with an empty Align reaches the protected result cloud.  Returns the
 * MSE, or -1 on an empty cloud. */
namespace {
struct CloudMSEProbe : registration::ICPBase {
    void Align() override {}
    void SetResult(pcl::PointCloud<pcl::PointXYZRGB>::Ptr c) { result_cloud_ = c; }
};
pcl::PointCloud<pcl::PointXYZRGB>::Ptr make_cloud(const float* xyz, size_t n) {
    pcl::PointCloud<pcl::PointXYZRGB>::Ptr c(new pcl::PointCloud<pcl::PointXYZRGB>());
    c->resize(n);
    for (size_t i = 0; i < n; ++i) {
        (*c)[i].x = xyz[3 * i];
        (*c)[i].y = xyz[3 * i + 1];
        (*c)[i].z = xyz[3 * i + 2];
    }
    return c;
}
}  // namespace

float ref_cloud_mse(const float* a, size_t na, const float* b, size_t nb) {
    try {
        CloudMSEProbe r;
        r.SetResult(make_cloud(a, na));
        r.SetTargetCloud(make_cloud(b, nb));
        return r.CloudMSE();
    } catch (const common::Exception&) {
        return -1.0f;
    }
}

/* ---- common::MSE::Compute (src/registration/registration_base.cc:160-240)
 * of coloured clouds p and q, through the reference's own class; out =
 * {geo p->q, geo q->p, Y.., Y.., U.., U.., V.., V..}.  Returns 0, or -1 when
 * the reference threw. */
int ref_mse_compute(const float* p, const uint8_t* prgb, size_t np, const float* q, const uint8_t* qrgb, size_t nq,
                    double* out) {
    auto coloured = [](const float* xyz, const uint8_t* rgb, size_t n) {
        pcl::PointCloud<pcl::PointXYZRGB>::Ptr c = make_cloud(xyz, n);
        for (size_t i = 0; i < n; ++i) {
            (*c)[i].r = rgb[3 * i];
            (*c)[i].g = rgb[3 * i + 1];
            (*c)[i].b = rgb[3 * i + 2];
        }
        return c;
    };
    try {
        common::MSE m;
        m.SetClouds(coloured(p, prgb, np), coloured(q, qrgb, nq));
        m.Compute();
        const std::pair<float, float> v[4] = {m.GetGeoMSEs(), m.GetYMSEs(), m.GetUMSEs(), m.GetVMSEs()};
        for (int k = 0; k < 4; ++k) {
            out[2 * k] = v[k].first;
            out[2 * k + 1] = v[k].second;
        }
        return 0;
    } catch (const common::Exception&) {
        return -1;
    }
}

/* ---- PatchFitting::Compute (src/patch/patch_fitting.cc:92-136, Split and
 * Clustering :138-381) with the reference configs' direct clustering: the
 * GoP's registered patches -> the fitting cloud.  srand(seed) first: the
 * reference draws its k-means seeds and empty-cluster replacements from the
 * process-wide rand().  Returns the fitting cloud's size (its xyz into
 * out[3 * cap]), or -1 when the reference threw, -2 when out is too small. */
long ref_fitting_cloud(int npatches, const float* const* xyz, const uint32_t* n, float clustering_ths,
                       float clustering_err_ths, int max_iter, unsigned seed, float* out, size_t cap) {
    try {
        patch::PatchFitting fit;
        auto prm = std::make_shared<common::PVVCParam_t>();
        prm->patch.clustering_ths = clustering_ths;
        prm->patch.clustering_err_ths = clustering_err_ths;
        prm->patch.max_iter = max_iter;
        prm->patch.split_method = common::DIRECT_CLUSTERING;
        fit.params_ = prm;
        for (int i = 0; i < npatches; ++i) {
            common::Patch pt;
            pt.cloud = make_cloud(xyz[i], n[i]);
            pt.index = 0;
            pt.timestamp = i;
            fit.source_patches_.emplace_back(pt);
        }
        fit.fitting_cloud_.reset(new pcl::PointCloud<pcl::PointXYZRGB>());
        srand(seed);
        fit.Compute();
        const auto& c = *fit.fitting_cloud_;
        if (c.size() > cap) return -2;
        for (size_t i = 0; i < c.size(); ++i) {
            out[3 * i] = c[i].x;
            out[3 * i + 1] = c[i].y;
            out[3 * i + 2] = c[i].z;
        }
        return (long)c.size();
    } catch (const common::Exception&) {
        return -1;
    }
}

int ref_change_slice_to_frame(const char* dir, const char* out_name) {
    try {
        io::ChangeSliceToFrame(dir, out_name);
        return 0;
    } catch (const common::Exception&) {
        return -1;
    }
}

}  // extern "C"
