// CPanel's result files (include/cpanel_io.h).  Host code only.
//
// The layout (labels, column widths, precisions, array names) is CPanel's, so that the
// files diff against the reference's own output: caseMgr::writeSummary/writeCase
// (CPanel/CPanelMgr.cpp:89-180), inputParams::print (CPanel/inputParams.cpp:227-318) and
// VTUfile::write (CPanel/VTUfile.cpp:20-147).  C++ streams are used with the same
// manipulators, so numbers are formatted exactly as the reference formats them.
#include <fstream>
#include <iomanip>
#include <new>
#include <ostream>
#include <string>

#include "../../include/cpanel_io.h"

namespace {

// a parameter list as inputParams::printVec prints it: "v " or "[a b c] "
void print_list(std::ostream& s, const double* v, int n) {
    if (n <= 0) return;
    if (n == 1) {
        s << v[0] << " ";
        return;
    }
    for (int i = 0; i < n; i++) {
        if (i == 0)
            s << "[" << v[i] << " ";
        else if (i == n - 1)
            s << v[i] << "] ";
        else
            s << v[i] << " ";
    }
}

void print_inputs(std::ostream& s, const cpg_cpout_inputs& in) {
    const int w = 28;
    auto flag = [&](const char* label, int on) {
        s << std::setw(w) << label << "-> " << (on ? "ON" : "OFF") << std::endl;
    };
    s << std::setw(w) << "Geometry File " << "-> " << (in.geom_file ? in.geom_file : "") << std::endl;
    s << std::setw(w) << "Reference Area " << "-> " << in.Sref << " ft^2" << std::endl;
    s << std::setw(w) << "Reference Span " << "-> " << in.bref << " ft" << std::endl;
    s << std::setw(w) << "Reference Chord " << "-> " << in.cref << " ft" << std::endl;
    s << std::setw(w) << "Center of Gravity " << "-> [" << in.cg[0] << " " << in.cg[1] << " " << in.cg[2] << "] ft"
      << std::endl;
    s << std::setw(w) << "Velocity " << "-> ";
    print_list(s, in.velocities, in.n_velocities);
    s << "ft/s" << std::endl;
    s << std::setw(w) << "Alpha " << "-> ";
    print_list(s, in.alphas, in.n_alphas);
    s << "degrees" << std::endl;
    s << std::setw(w) << "Beta " << "-> ";
    print_list(s, in.betas, in.n_betas);
    s << "degrees" << std::endl;
    s << std::setw(w) << "Mach # " << "-> ";
    print_list(s, in.machs, in.n_machs);
    s << std::endl;
    flag("Subsonic HOM ", in.subsonic_hom);
    flag("Surface Streamlines ", in.surface_streamlines);
    flag("Stability Derivatives ", in.stability_derivatives);
    flag("Write Inf Coeff to File ", in.write_inf_coeff);
    flag("Vortex Particle Wake ", in.vortex_particles);
    flag("Accelerate Code ", in.accelerate_code);
    flag("Unsteady Mode ", in.unsteady);
}

void print_case(std::ostream& s, int number, const cpg_cpout_case& c) {
    const int sp[4] = {11, 7, 8, 8};  // Velocity, Mach, Alpha, Beta columns
    s << std::endl;
    s << std::setprecision(3);
    s << "---Case #" << number << "---" << std::endl;
    s << "\n\t--Flow Conditions--\n" << std::endl;
    s << "\t\t" << std::setw(sp[0]) << "Velocity" << std::setw(sp[1]) << "Mach" << std::setw(sp[2]) << "Alpha"
      << std::setw(sp[3]) << "Beta" << "\n";
    s << "\t\t" << std::setw(sp[0]) << c.flow.V << std::setw(sp[1]) << c.flow.mach << std::setw(sp[2]) << c.flow.alpha
      << std::setw(sp[3]) << c.flow.beta << "\n";
    s << std::setprecision(5);
    s << "\n\t--Force Coefficients--\n" << std::endl;
    s << "\t\t-Trefftz Plane-" << std::endl;
    s << "\t\t\tCL = " << c.CL << "\tCDi = " << c.CDi << std::endl;
    s << "\n\t\t-Surface Integrated Force Coefficients-" << std::endl;
    s << "\t\t\t" << std::setw(15) << "Body Axis" << std::setw(10) << "CN" << std::setw(10) << "CA" << std::setw(10)
      << "CY" << std::endl;
    s << "\t\t\t" << std::setw(15) << " " << std::setw(10) << c.Fbody[2] << std::setw(10) << c.Fbody[0]
      << std::setw(10) << c.Fbody[1] << std::endl;
    s << "\t\t\t" << std::setw(15) << "Wind Axis" << std::setw(10) << "CL" << std::setw(10) << "CD" << std::setw(10)
      << "CY" << std::endl;
    s << "\t\t\t" << std::setw(15) << " " << std::setw(10) << c.Fwind[2] << std::setw(10) << c.Fwind[0]
      << std::setw(10) << c.Fwind[1] << std::endl;
    s << "\n\t--Moment Coefficients--\n" << std::endl;
    s << "\t\t" << std::setw(12) << "Cm (pitch)" << std::setw(12) << "Cl (roll)" << std::setw(12) << "Cn (yaw)"
      << std::endl;
    s << "\t\t" << std::setw(12) << c.CM[1] << std::setw(12) << c.CM[0] << std::setw(12) << c.CM[2] << std::endl;
    if (c.has_stability) {
        const cpg_stability& d = c.stability;
        s << "\n\t--Stability Derivatives--\n" << std::endl;
        s << "\t\t" << std::setw(12) << "CL_alpha" << std::setw(12) << "CY_alpha" << std::setw(12) << "Cm_alpha"
          << std::setw(12) << "Cl_alpha" << std::setw(12) << "Cn_alpha" << std::endl;
        s << "\t\t" << std::setw(12) << d.dF_dAlpha[2] << std::setw(12) << d.dF_dAlpha[1] << std::setw(12)
          << d.dM_dAlpha[1] << std::setw(12) << d.dM_dAlpha[0] << std::setw(12) << d.dM_dAlpha[2] << std::endl;
        s << "\t\t" << std::setw(12) << "CL_beta" << std::setw(12) << "CY_beta" << std::setw(12) << "Cm_beta"
          << std::setw(12) << "Cl_beta" << std::setw(12) << "Cn_beta" << std::endl;
        s << "\t\t" << std::setw(12) << d.dF_dBeta[2] << std::setw(12) << d.dF_dBeta[1] << std::setw(12)
          << d.dM_dBeta[1] << std::setw(12) << d.dM_dBeta[0] << std::setw(12) << d.dM_dBeta[2] << std::endl;
        s << "\n\n" << std::endl;
    }
}

// one DataArray of doubles: rows x cols, tab after every value, newline per row
void print_doubles(std::ostream& f, const char* name, const double* a, int64_t rows, int cols, int64_t stride = 0,
                   int64_t offset = 0) {
    f << "\t\t\t\t<DataArray type=\"Float64\" Name=\"" << name << "\" NumberOfComponents=\"" << cols
      << "\" Format=\"ascii\">\n";
    const int64_t st = stride ? stride : cols;
    for (int64_t i = 0; i < rows; i++) {
        for (int j = 0; j < cols; j++) f << a[i * st + offset + j] << "\t";
        f << "\n";
    }
    f << "\t\t\t\t</DataArray>\n";
}

}  // namespace

extern "C" {

int cpg_write_cpout(const char* path, const cpg_cpout_inputs* in, const cpg_cpout_case* cases, int n) {
    if (!path || !in || (n > 0 && !cases) || n < 0) return CPG_E_INVALID;
    try {
        std::ofstream out(path);
        if (!out) return CPG_E_INVALID;
        out << "-----------INPUTS-----------\n\n";
        print_inputs(out, *in);
        out << "\n\n";
        out << "-----------RESULTS-----------\n\n";
        out << std::left << std::fixed;
        for (int i = 0; i < n; i++) print_case(out, i + 1, cases[i]);
        out.close();
        return out ? CPG_OK : CPG_E_INVALID;
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

int cpg_write_surface_vtu(const char* path, const double* nodes, int64_t nn, const int64_t* tris, int64_t n,
                          const double* mu, const double* sigma, const double* phi, const double* vel,
                          const double* cp, const double* bez, const double* centers) {
    if (!path || !nodes || !tris || nn <= 0 || n <= 0 || !mu || !sigma || !phi || !vel || !cp || !bez || !centers)
        return CPG_E_INVALID;
    for (int64_t i = 0; i < 3 * n; i++)
        if (tris[i] < 0 || tris[i] >= nn) return CPG_E_INVALID;
    try {
        std::ofstream f(path);
        if (!f) return CPG_E_INVALID;
        f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        f << "\t<UnstructuredGrid>\n";
        f << "\t\t<Piece NumberOfPoints=\"" << nn << "\" NumberOfCells=\"" << n << "\">\n";
        f << "\t\t\t<CellData Scalars=\"scalars\">\n";
        print_doubles(f, "Doublet Strengths", mu, n, 1);
        print_doubles(f, "Source Strengths", sigma, n, 1);
        print_doubles(f, "Velocity Potential", phi, n, 1);
        print_doubles(f, "Velocity", vel, n, 3);
        print_doubles(f, "Cp", cp, n, 1);
        print_doubles(f, "bezNormals", bez, n, 3);
        print_doubles(f, "xPosition", centers, n, 1, 3, 0);
        print_doubles(f, "yPosition", centers, n, 1, 3, 1);
        print_doubles(f, "zPostition", centers, n, 1, 3, 2);  // the reference's spelling
        f << "\t\t\t</CellData>\n";
        f << "\t\t\t<Points>\n";
        print_doubles(f, "Position", nodes, nn, 3);
        f << "\t\t\t</Points>\n";
        f << "\t\t\t<Cells>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << tris[3 * i] << "\t" << tris[3 * i + 1] << "\t" << tris[3 * i + 2] << "\t\n";
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << (i + 1) * 3 << "\t\n";
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << 5 << "\t\n";  // VTK_TRIANGLE
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t</Cells>\n";
        f << "\t\t</Piece>\n";
        f << "\t</UnstructuredGrid>\n";
        f << "</VTKFile>\n";
        f.close();
        return f ? CPG_OK : CPG_E_INVALID;
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

int cpg_write_wake_vtu(const char* path, const double* nodes, int64_t nn, const int64_t* tris, int64_t n,
                       const double* mu, const double* phi) {
    if (!path || !nodes || !tris || nn <= 0 || n <= 0 || !mu || !phi) return CPG_E_INVALID;
    for (int64_t i = 0; i < 3 * n; i++)
        if (tris[i] < 0 || tris[i] >= nn) return CPG_E_INVALID;
    try {
        std::ofstream f(path);
        if (!f) return CPG_E_INVALID;
        f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        f << "\t<UnstructuredGrid>\n";
        f << "\t\t<Piece NumberOfPoints=\"" << nn << "\" NumberOfCells=\"" << n << "\">\n";
        f << "\t\t\t<CellData Scalars=\"scalars\">\n";
        print_doubles(f, "Doublet Strengths", mu, n, 1);
        print_doubles(f, "Velocity Potential", phi, n, 1);
        f << "\t\t\t</CellData>\n";
        f << "\t\t\t<Points>\n";
        print_doubles(f, "Position", nodes, nn, 3);
        f << "\t\t\t</Points>\n";
        f << "\t\t\t<Cells>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << tris[3 * i] << "\t" << tris[3 * i + 1] << "\t" << tris[3 * i + 2] << "\t\n";
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << (i + 1) * 3 << "\t\n";
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < n; i++) f << 5 << "\t\n";  // VTK_TRIANGLE
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t</Cells>\n";
        f << "\t\t</Piece>\n";
        f << "\t</UnstructuredGrid>\n";
        f << "</VTKFile>\n";
        f.close();
        return f ? CPG_OK : CPG_E_INVALID;
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

int cpg_write_volume_vtu(const char* path, const double* pts, int64_t np, const int64_t* cells, int64_t nc,
                         const double* vel, const double* cp) {
    if (!path || !pts || !cells || np <= 0 || nc <= 0 || !vel || !cp) return CPG_E_INVALID;
    for (int64_t i = 0; i < 8 * nc; i++)
        if (cells[i] < 0 || cells[i] >= np) return CPG_E_INVALID;
    try {
        std::ofstream f(path);
        if (!f) return CPG_E_INVALID;
        f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        f << "\t<UnstructuredGrid>\n";
        f << "\t\t<Piece NumberOfPoints=\"" << np << "\" NumberOfCells=\"" << nc << "\">\n";
        f << "\t\t\t<CellData Scalars=\"scalars\">\n";
        print_doubles(f, "Velocity", vel, nc, 3);
        print_doubles(f, "Cp", cp, nc, 1);
        f << "\t\t\t</CellData>\n";
        f << "\t\t\t<Points>\n";
        print_doubles(f, "Position", pts, np, 3);
        f << "\t\t\t</Points>\n";
        f << "\t\t\t<Cells>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < nc; i++) {
            for (int q = 0; q < 8; q++) f << cells[8 * i + q] << "\t";
            f << "\n";
        }
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < nc; i++) f << (i + 1) * 8 << "\t\n";
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n";
        for (int64_t i = 0; i < nc; i++) f << 11 << "\t\n";  // VTK_VOXEL
        f << "\t\t\t\t</DataArray>\n";
        f << "\t\t\t</Cells>\n";
        f << "\t\t</Piece>\n";
        f << "\t</UnstructuredGrid>\n";
        f << "</VTKFile>\n";
        f.close();
        return f ? CPG_OK : CPG_E_INVALID;
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

int cpg_write_streamlines_vtu(const char* path, const double* pts, const double* vel, const int32_t* counts,
                              int n_lines, int max_points) {
    if (!path || n_lines < 0 || max_points < 0 || (n_lines > 0 && !counts)) return CPG_E_INVALID;
    for (int i = 0; i < n_lines; i++)
        if (counts[i] < 0 || counts[i] > max_points) return CPG_E_INVALID;
    if (n_lines > 0 && max_points > 0 && (!pts || !vel)) return CPG_E_INVALID;
    try {
        std::ofstream f(path);
        if (!f) return CPG_E_INVALID;
        f << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        f << "\t<UnstructuredGrid>\n";
        for (int i = 0; i < n_lines; i++) {  // one piece per line, cells (j, j + 1)
            const int64_t np = counts[i], nc = np > 0 ? np - 1 : 0;
            const int64_t o = (int64_t)i * max_points * 3;
            f << "\t\t<Piece NumberOfPoints=\"" << np << "\" NumberOfCells=\"" << nc << "\">\n";
            f << "\t\t\t<PointData Scalars=\"scalars\">\n";
            print_doubles(f, "Velocity", vel + o, np, 3);
            f << "\t\t\t</PointData>\n";
            f << "\t\t\t<Points>\n";
            print_doubles(f, "Position", pts + o, np, 3);
            f << "\t\t\t</Points>\n";
            f << "\t\t\t<Cells>\n";
            f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n";
            for (int64_t j = 0; j < nc; j++) f << j << "\t" << j + 1 << "\t\n";
            f << "\t\t\t\t</DataArray>\n";
            f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n";
            for (int64_t j = 0; j < nc; j++) f << (j + 1) * 2 << "\t\n";
            f << "\t\t\t\t</DataArray>\n";
            f << "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n";
            for (int64_t j = 0; j < nc; j++) f << 3 << "\t\n";  // VTK_LINE
            f << "\t\t\t\t</DataArray>\n";
            f << "\t\t\t</Cells>\n";
            f << "\t\t</Piece>\n";
        }
        f << "\t</UnstructuredGrid>\n";
        f << "</VTKFile>\n";
        f.close();
        return f ? CPG_OK : CPG_E_INVALID;
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

int cpg_write_spanwise_csv(const char* path, const double* y2b, const double* cl, const double* cdi, int n) {
    if (!path || n < 0 || (n > 0 && (!y2b || !cl || !cdi))) return CPG_E_INVALID;
    std::ofstream f(path);
    if (!f) return CPG_E_INVALID;
    // a header line, then one row per station in the stream's default format (six significant digits)
    f << "2y/b,Cl,Cdi" << std::endl;
    for (int j = 0; j < n; j++) f << y2b[j] << "," << cl[j] << "," << cdi[j] << std::endl;
    f.close();
    return f ? CPG_OK : CPG_E_INVALID;
}

}  // extern "C"
