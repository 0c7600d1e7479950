// C entry points around the reference's own FacesNMF image loader, for the tests.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file in the
// container that holds the reference tree.  The reference's loader is two
// member functions of an MFC dialog (src/examples/FacesNMF/FacesNMFDlg.cpp:
// FolderHasImages at 313-347 and LoadImage at 409-472); the build recipe
// copies those two function definitions, unchanged, out of that file into the
// git-ignored oracle/_ref/faces_dlg_methods.inc, and this file gives them the
// few MFC names they use (CString, CFile::GetStatus, a check box, the error
// report) as plain C++ stand-ins, so the reference's own header parsing,
// read() offset and float histogram equalisation run here as written.  The
// reference joins folder and file name with a backslash, so callers pass a
// folder whose backslash-joined names exist (the recipe makes such links).
//
// The library that results (oracle/_ref/libfaces_ref.so) is never part of the
// product: it pins the restatement in oracle/faces.py and generates the
// golden data of tests/golden/make_faces_golden.py.
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <sys/stat.h>

#include "definitions.h"   // reference src/cuda/definitions.h: cudafloat = float
#include "Matrix.h"        // generated copy of src/examples/FacesNMF/Matrix.h (see build.py)
#include "HostArray.h"     // reference src/memory/HostArray.h

using namespace std;
using namespace GPUMLib;

namespace {

struct CString {
    std::string s;
};
ostream &operator<<(ostream &o, const CString &c) { return o << c.s; }

struct CFileStatus {};
struct CFile {
    static bool GetStatus(const char *path, CFileStatus &) {
        struct stat st;
        return stat(path, &st) == 0;
    }
};

const int BST_CHECKED = 1;
struct CheckBox {
    int state = BST_CHECKED;   // FacesNMFDlg.cpp:138 checks it when the dialog opens
    int GetCheck() const { return state; }
};

class CFacesNMFDlg {
public:
    bool errorsLoadingImages = false, errorsLoadingImagesTest = false;
    int imageWidth = 0, imageHeight = 0;
    CheckBox checkHistogram;
    int errors = 0;
    void ErrorLoadingImage(const char *) { errors++; }
    bool FolderHasImages(CString &folder, int &numberImages, int &imageWidth, int &imageHeight);
    bool LoadImage(CString &folder, int imageNumber, Matrix<cudafloat> &V);
};

#include "faces_dlg_methods.inc"   // the two reference definitions, copied verbatim

}  // namespace

// FolderHasImages: returns 1 when the folder holds images, with their count and size.
extern "C" int ref_faces_scan(const char *folder, int *count, int *width, int *height) {
    CFacesNMFDlg dlg;
    CString f{folder};
    int c = 0, w = 0, h = 0;
    bool ok = dlg.FolderHasImages(f, c, w, h);
    *count = c;
    *width = w;
    *height = h;
    return ok ? 1 : 0;
}

// LoadImage for images 0..count-1 into V (pixels x count, column-major).  ok[i]
// receives LoadImage's return value; columns of images that failed keep what
// the reference left there (V is zeroed first).  Returns the number of failures.
extern "C" int ref_faces_load(const char *folder, int count, int width, int height, int equalize, float *V,
                              int *ok) {
    CFacesNMFDlg dlg;
    dlg.imageWidth = width;
    dlg.imageHeight = height;
    dlg.checkHistogram.state = equalize ? BST_CHECKED : 0;
    CString f{folder};
    const int pixels = width * height;
    Matrix<cudafloat> M(pixels, count, ColumnMajor);   // as HostNMF's V (HostNMF.h:250)
    std::memset(M.Pointer(), 0, sizeof(float) * (size_t)pixels * count);
    int failed = 0;
    for (int i = 0; i < count; i++) {
        bool good = dlg.LoadImage(f, i, M);
        if (ok) ok[i] = good ? 1 : 0;
        if (!good) failed++;
    }
    std::memcpy(V, M.Pointer(), sizeof(float) * (size_t)pixels * count);
    return failed;
}
