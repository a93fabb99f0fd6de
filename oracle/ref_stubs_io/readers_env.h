// Forced in ahead of Source/sc_readdata.cpp (test oracle only): a stand-in for
// the console program's widImage (image extents, data and meta information,
// as the readers use them) under the real header's include guard, so that
// the reference's own readers compile and run without Qt.
#ifndef CS_IO_READERS_ENV_H
#define CS_IO_READERS_ENV_H
#define WIDIMAGE_H
#define NOHDF5
#define CONSOLENPROG
#include <cmath>
#include <vector>
#include "QDebug"
#include "QFile"
#include "QHash"
#include "QString"
#include "QVector"
// the reference's image index (widimage.h): x inner, y outer
#define XY2IDX(X0, X1, Y0, Y1, x, y) ((-X0 + (x)) + (X1 - X0) * (-Y0 + (y)))
class widImage {
public:
    typedef struct {
        double wavelen;
        double distance;
        double pixWidthX, pixWidthY;
        int pixelX, pixelY;
        int centerX, centerY;
        QString filePath;
        int isValid;
    } _fileInfos;
    int minX = 0, maxX = 0, minY = 0, maxY = 0;
    QVector<double> data;
    QString title;
    std::vector<QString> metaKeys, metaVals;
    _fileInfos fileInfos{};
    void addMetaInfo(QString key, QString val) {
        metaKeys.push_back(key);
        metaVals.push_back(val);
    }
    int setData(int x0, int x1, int y0, int y1, double *d) {
        minX = x0;
        maxX = x1;
        minY = y0;
        maxY = y1;
        data.assign(d, d + (size_t)(x1 - x0) * (size_t)(y1 - y0));
        return 0;
    }
    const double *dataPtr() { return data.constData(); }
    double xmin() { return minX; }
    double xmax() { return maxX; }
    double ymin() { return minY; }
    double ymax() { return maxY; }
    int myWidth() { return maxX - minX; }
    int myHeight() { return maxY - minY; }
    double getData(int x, int y) { return data[(size_t)XY2IDX(minX, maxX, minY, maxY, x, y)]; }
    _fileInfos *getFileInfos() { return &fileInfos; }
};
#endif
