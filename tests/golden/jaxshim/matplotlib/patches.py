class RegularPolygon:
    pass
