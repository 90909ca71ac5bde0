// Mat-8.3.1/QR/QR.h:5 includes "__HouseHolder_Blocked.h" but the file is named
// QR/__Householder_Blocked.h (resolves only on case-insensitive file systems).
#include <QR/__Householder_Blocked.h>
