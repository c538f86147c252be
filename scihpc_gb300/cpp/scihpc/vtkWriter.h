// vtkWriter.h -- legacy VTK (STRUCTURED_POINTS, big-endian binary CELL_DATA) output of
// fields (reference scihpc/vtkWriter.h:14-37).  Fields owned by a GPU session are
// downloaded before they are written.
#ifndef SCIHPC_GB300_VTKWRITER_H
#define SCIHPC_GB300_VTKWRITER_H

#include <fstream>
#include <string>

#include "global.h"
#include "scalar_data.h"
#include "structured_grid.h"
#include "vector_data.h"

class vtkWriter {
public:
    vtkWriter(structured_grid *_geo, std::string _filename);

    structured_grid *grid;
    std::string filename;
    std::ofstream file;

    void create(unsigned int id);
    void add_scalar(scalar_data *data, const std::string &name);
    void add_scalar(DataType ***_data, scalar_data *data, const std::string &name);
    void add_vector(vector_data *data, const std::string &name);
    void add_vector(DataType ***u, DataType ***v, DataType ***w, vector_data *data, const std::string &name);
    void close();
};

#endif
